// Contraction engine: C[ic] = alpha A[ia] B[ib] + beta C[ic] on dense
// column-major device tensors.
//
// Each call becomes at most one permutation per operand plus one GEMM.  The
// free indices of A (M), of B (N) and the summed indices (K) may each be
// ordered as they appear in either operand or in C; the planner tries every
// combination and keeps the one that moves the fewest bytes, so operands whose
// indices already form [M|K] / [K|M] blocks are used in place (op N / op T)
// and C is written directly when its indices form [M|N] (or [N|M], by
// computing the transposed product).
#include <cstring>
#include <string>

#include "internal.hpp"

namespace gbcc {
namespace {

struct Plan {
  std::string m, n, k;   // index orders
  bool permA = false, permB = false, permC = false;
  bool ta = false, tb = false, swap = false;
  double cost = 0;
};

std::string restrict_to(const std::string &order, const std::string &set) {
  std::string r;
  for (char c : order)
    if (set.find(c) != std::string::npos) r += c;
  return r;
}

int64_t prod(const std::string &s, const int64_t *len) {
  int64_t p = 1;
  for (char c : s) p *= len[(unsigned char)c];
  return p;
}

}  // namespace

void assign(Context &ctx, double alpha, const Ten &A, const char *ia,
            double beta, const Ten &C, const char *ic) {
  const int n = (int)std::strlen(ia);
  require(n == A.order && (int)std::strlen(ic) == C.order && n == C.order,
          std::string("assign: bad index strings ") + ia + " -> " + ic);
  int perm[6];
  for (int q = 0; q < n; ++q) {
    const char *f = std::strchr(ia, ic[q]);
    require(f != nullptr, "assign: index not found");
    perm[q] = (int)(f - ia);
  }
  Ten dst = C;
  permute(ctx, A, perm, alpha, beta, dst);
}

void contract(Context &ctx, double alpha, const Ten &A, const char *ia,
              const Ten &B, const char *ib, double beta, const Ten &C,
              const char *ic, int precision) {
  const std::string sa(ia), sb(ib), sc(ic);
  require((int)sa.size() == A.order && (int)sb.size() == B.order &&
              (int)sc.size() == C.order,
          "contract: index string / order mismatch: " + sa + "," + sb + "->" +
              sc);
  int64_t len[256];
  for (auto &l : len) l = -1;
  auto bind = [&](const std::string &s, const Ten &t) {
    for (size_t d = 0; d < s.size(); ++d) {
      const unsigned char c = (unsigned char)s[d];
      if (len[c] < 0) len[c] = t.lens[d];
      require(len[c] == t.lens[d],
              "contract: length mismatch for index " + std::string(1, s[d]) +
                  " in " + sa + "," + sb + "->" + sc);
    }
  };
  bind(sa, A);
  bind(sb, B);
  bind(sc, C);
  std::string M, N, K;
  for (char c : sa) {
    const bool inB = sb.find(c) != std::string::npos;
    const bool inC = sc.find(c) != std::string::npos;
    require(!(inB && inC), "contract: batch indices are not supported");
    require(inB || inC, "contract: index summed in one operand only");
    if (inC) M += c; else K += c;
  }
  for (char c : sb) {
    const bool inA = sa.find(c) != std::string::npos;
    const bool inC = sc.find(c) != std::string::npos;
    require(inA || inC, "contract: index summed in one operand only");
    if (inC) N += c;
  }
  for (char c : sc)
    require(sa.find(c) != std::string::npos || sb.find(c) != std::string::npos,
            "contract: output index not in any operand");
  const int64_t sM = prod(M, len), sN = prod(N, len), sK = prod(K, len);

  // candidate orders
  const std::string mo[2] = {restrict_to(sa, M), restrict_to(sc, M)};
  const std::string no[2] = {restrict_to(sb, N), restrict_to(sc, N)};
  const std::string ko[2] = {restrict_to(sa, K), restrict_to(sb, K)};
  Plan best;
  best.cost = 1e300;
  for (const auto &m : mo)
    for (const auto &nn : no)
      for (const auto &k : ko) {
        Plan p;
        p.m = m;
        p.n = nn;
        p.k = k;
        if (sa == m + k) p.ta = false;
        else if (sa == k + m) p.ta = true;
        else { p.permA = true; p.ta = false; p.cost += 2.0 * A.size(); }
        if (sb == k + nn) p.tb = false;
        else if (sb == nn + k) p.tb = true;
        else { p.permB = true; p.tb = false; p.cost += 2.0 * B.size(); }
        if (sc == m + nn) p.swap = false;
        else if (sc == nn + m) p.swap = true;
        else {
          p.permC = true;
          p.cost += 2.0 * C.size() + (beta != 0.0 ? 1.0 * C.size() : 0.0);
        }
        if (p.cost < best.cost) best = p;
      }
  const Plan &p = best;
  // operand A as a [M,K] (ta=0) or [K,M] (ta=1) matrix
  const double *pa = A.p;
  int64_t lda = p.ta ? sK : sM;
  DBuf ta_buf, tb_buf, tc_buf;
  if (p.permA) {
    ta_buf.alloc(ctx, sizeof(double) * A.size());
    Ten t = A;
    t.p = ta_buf.as<double>();
    const std::string o = p.m + p.k;
    for (size_t d = 0; d < o.size(); ++d) t.lens[d] = len[(unsigned char)o[d]];
    assign(ctx, 1.0, A, sa.c_str(), 0.0, t, o.c_str());
    pa = t.p;
    lda = sM;
  }
  const double *pb = B.p;
  int64_t ldb = p.tb ? sN : sK;
  if (p.permB) {
    tb_buf.alloc(ctx, sizeof(double) * B.size());
    Ten t = B;
    t.p = tb_buf.as<double>();
    const std::string o = p.k + p.n;
    for (size_t d = 0; d < o.size(); ++d) t.lens[d] = len[(unsigned char)o[d]];
    assign(ctx, 1.0, B, sb.c_str(), 0.0, t, o.c_str());
    pb = t.p;
    ldb = sK;
  }
  double *pc = C.p;
  double gbeta = beta;
  if (p.permC) {
    tc_buf.alloc(ctx, sizeof(double) * C.size());
    pc = tc_buf.as<double>();
    gbeta = 0.0;
  }
  if (!p.swap) {
    gemm(ctx, p.ta, p.tb, sM, sN, sK, alpha, pa, lda, pb, ldb, gbeta, pc, sM,
         1, 0, 0, 0, precision);
  } else {
    // C^T[N,M] = op(B)^T op(A)^T
    gemm(ctx, !p.tb, !p.ta, sN, sM, sK, alpha, pb, ldb, pa, lda, gbeta, pc,
         sN, 1, 0, 0, 0, precision);
  }
  if (p.permC) {
    Ten t = C;
    t.p = pc;
    const std::string o = p.m + p.n;
    for (size_t d = 0; d < o.size(); ++d) t.lens[d] = len[(unsigned char)o[d]];
    assign(ctx, 1.0, t, o.c_str(), beta, C, sc.c_str());
  }
}

}  // namespace gbcc
