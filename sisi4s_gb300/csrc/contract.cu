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
#include <cstdio>
#include <cstring>
#include <memory>
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

// Offsets of the index group g (mixed radix, first index fastest) inside a
// tensor with index string s, as v s0 or, for two runs of indices whose
// strides chain, (v % l) s0 + (v / l) s1.  False for three or more runs.
bool group_offsets(const std::string &s, const std::string &g, const int64_t *len,
                   int64_t &s0, unsigned &l, int64_t &s1) {
  int64_t st[256] = {};
  int64_t acc = 1;
  for (char c : s) {
    st[(unsigned char)c] = acc;
    acc *= len[(unsigned char)c];
  }
  int64_t rs[2] = {0, 0}, rl[2] = {1, 1};
  int n = 0;
  for (char c : g) {
    const int64_t sc = st[(unsigned char)c], lc = len[(unsigned char)c];
    if (lc == 1) continue;  // a length-1 index moves nothing
    if (n > 0 && rs[n - 1] * rl[n - 1] == sc) {
      rl[n - 1] *= lc;
      continue;
    }
    if (n == 2) return false;
    rs[n] = sc;
    rl[n] = lc;
    ++n;
  }
  s0 = n > 0 ? rs[0] : 0;
  l = 0;
  s1 = 0;
  if (n == 2) {
    if (rl[0] >= (1LL << 31)) return false;
    l = (unsigned)rl[0];
    s1 = rs[1];
  }
  return true;
}

}  // namespace

// The plan of contract() with emulated panels, for a contraction with a
// registered constant operand: the constant operand's panels (after its
// permutation, if the plan has one) are split once per layout and role and
// kept in the context; the other operand is permuted and split as usual.
// The digits are those the plain route would produce, so the result is the
// same bit for bit.
// With a batch index z (nz entries, the last index of A, B and C; sa, sb,
// sc the index strings without it) every operand is a family of nz panels
// and the product one batched launch.
void contract_cached(Context &ctx, double alpha, const Ten &A, const std::string &sa,
                     const Ten &B, const std::string &sb, double beta, const Ten &C,
                     const std::string &sc, const std::string &m, const std::string &n,
                     const std::string &k, bool permA, bool ta, bool permB, bool tb,
                     bool permC, bool swap, const int64_t *len, char z, int64_t nz) {
  const int64_t sM = prod(m, len), sN = prod(n, len), sK = prod(k, len);
  const std::string zs = z ? std::string(1, z) : std::string();
  // panels of one operand: tensor T (index string st), GEMM order `order`
  // (permuted into it when perm), matrix with `rows` rows, element (r, q) at
  // r*rs + q*ks of the GEMM-ready buffer
  auto panels = [&](const Ten &T, const std::string &st, bool perm, const std::string &order,
                    const std::string &rg, bool role_a, int64_t rows, int64_t rs, int64_t ks)
      -> std::shared_ptr<EmuPanels> {
    const bool constant =
        ctx.use_panel_cache && ctx.is_constant(T.p, sizeof(double) * T.size());
    // an operand unchanged for this residual evaluation: its panels of this
    // layout and role, if already split, are reused
    std::string fkey;
    if (!constant && ctx.is_frozen(T.p, sizeof(double) * T.size())) {
      char buf[64];
      std::snprintf(buf, sizeof buf, "%p", (const void *)T.p);
      fkey = std::string(buf) + "|" + st + "|" + rg + "|" + k + "|" + (role_a ? "A" : "B") +
             "|" + std::to_string(rows) + "|" + std::to_string(nz) + "|" +
             std::to_string(ctx.emu_slices);
      auto it = ctx.frozen_panels.find(fkey);
      if (it != ctx.frozen_panels.end()) return it->second;
    }
    auto keep = [&](std::shared_ptr<EmuPanels> P) {
      const size_t b = P->panels.bytes() + P->exps.bytes();
      if (!fkey.empty() && ctx.frozen_bytes + b <= Context::FROZEN_PANEL_LIMIT) {
        ctx.frozen_panels[fkey] = P;
        ctx.frozen_bytes += b;
      }
      return P;
    };
    if (perm && !constant) {
      // an operand that changes from call to call is read in place when its
      // row indices (rg) and K indices each form at most two runs, one of
      // them contiguous; its digits are those of the permuted copy
      int64_t r0, r1, k0, k1;
      unsigned rl, kl;
      if (group_offsets(st, rg, len, r0, rl, r1) && group_offsets(st, k, len, k0, kl, k1) &&
          (r0 == 1 || k0 == 1) && rows < (1LL << 31) && sK < (1LL << 31)) {
        IdxMap mp;
        mp.rl = rl;
        mp.rs1 = r1;
        mp.kl = kl;
        mp.ks1 = k1;
        return keep(std::make_shared<EmuPanels>(
            emu_split(ctx, role_a, T.p, rows, sK, r0, k0, (int)nz, rows * sK, mp)));
      }
    }
    std::string key;
    if (constant) {
      char buf[64];
      std::snprintf(buf, sizeof buf, "%p", (const void *)T.p);
      key = std::string(buf) + "|" + st + ">" + order + "|" + (role_a ? "A" : "B") + "|" +
            std::to_string(rows) + "|" + std::to_string(rs) + "|" + std::to_string(ks) +
            "|" + std::to_string(ctx.emu_slices) + "|" + std::to_string(nz);
      auto it = ctx.panel_cache.find(key);
      if (it != ctx.panel_cache.end()) return it->second.panels;
    }
    const double *base = T.p;
    OTen tmp;
    if (perm) {
      tmp = OTen(ctx, {T.size()});
      Ten t = T;
      t.p = tmp.p();
      const std::string oz = order + zs;
      for (size_t d = 0; d < oz.size(); ++d) t.lens[d] = len[(unsigned char)oz[d]];
      assign(ctx, 1.0, T, (st + zs).c_str(), 0.0, t, oz.c_str());
      base = t.p;
    }
    auto P = std::make_shared<EmuPanels>(
        emu_split(ctx, role_a, base, rows, sK, rs, ks, (int)nz, rows * sK));
    if (constant) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      const size_t bytes = P->panels.bytes() + P->exps.bytes();
      // never keep buffers allocated inside a stream capture
      if (cudaStreamIsCapturing(ctx.stream, &cs) == cudaSuccess &&
          cs == cudaStreamCaptureStatusNone &&
          ctx.panel_cache_bytes + bytes <= Context::PANEL_CACHE_LIMIT) {
        ctx.panel_cache[key] = {T.p, P, bytes};
        ctx.panel_cache_bytes += bytes;
      }
    }
    return keep(P);
  };
  // The output is written in place through an index map when its row and
  // column indices each form at most two runs of C and one of the groups
  // starts contiguous; that group becomes the kernel's rows (a coalesced
  // write-out), M or, for the transposed product, N.
  bool sw = swap;
  OutMap cmap{};
  if (permC) {
    auto group_map = [&](const std::string &g, int64_t cnt, int64_t &l0, int64_t &s0,
                         int64_t &s1) {
      int64_t a0, a1;
      unsigned l;
      if (!group_offsets(sc, g, len, a0, l, a1)) return false;
      l0 = l ? (int64_t)l : cnt;  // one run: the whole range at the first level
      s0 = a0;
      s1 = l ? a1 : 0;
      return cnt < (1LL << 31);
    };
    int64_t ml0, ms0, ms1, nl0, ns0, ns1;
    if (group_map(m, sM, ml0, ms0, ms1) && group_map(n, sN, nl0, ns0, ns1)) {
      if (ms0 == 1) {
        sw = false;
        cmap = OutMap{ml0, ms0, ms1, nl0, ns0, ns1};
      } else if (ns0 == 1) {
        sw = true;
        cmap = OutMap{nl0, ns0, ns1, ml0, ms0, ms1};
      }
    }
  }
  // op(A)(m, k): from A's buffer in order m+k (ta = 0) or k+m (ta = 1)
  const std::string oa = permA ? m + k : sa;
  const bool tA = permA ? false : ta;
  const int64_t lda = tA ? sK : sM;
  // op(B)(k, n): order k+n (tb = 0) or n+k (tb = 1)
  const std::string ob = permB ? k + n : sb;
  const bool tB = permB ? false : tb;
  const int64_t ldb = tB ? sN : sK;
  // kernel roles: C = A_role (rows M) x B_role (rows N)^T, or the transposed
  // product when the plan computes C^T
  auto PA = panels(A, sa, permA, oa, m, !sw, sM, tA ? lda : 1, tA ? 1 : lda);
  auto PB = panels(B, sb, permB, ob, n, sw, sN, tB ? 1 : ldb, tB ? ldb : 1);
  if (cmap.ml0 > 0) {
    const EmuPanels &rows = sw ? *PB : *PA, &cols = sw ? *PA : *PB;
    if (nz > 1) emu_gemm_panels_batched(ctx, rows, cols, (int)nz, alpha, beta, C.p, 0, sM * sN, cmap);
    else emu_gemm_panels_mapped(ctx, rows, 0, cols, 0, alpha, beta, C.p, cmap);
    return;
  }
  double *pc = C.p;
  double gbeta = beta;
  OTen tc;
  if (permC) {
    tc = OTen(ctx, {C.size()});
    pc = tc.p();
    gbeta = 0.0;
  }
  if (nz > 1) {
    if (!swap) emu_gemm_panels_batched(ctx, *PA, *PB, (int)nz, alpha, gbeta, pc, sM, sM * sN);
    else emu_gemm_panels_batched(ctx, *PB, *PA, (int)nz, alpha, gbeta, pc, sN, sM * sN);
  } else if (!swap) {
    emu_gemm_panels(ctx, *PA, 0, *PB, 0, alpha, gbeta, pc, sM);
  } else {
    emu_gemm_panels(ctx, *PB, 0, *PA, 0, alpha, gbeta, pc, sN);
  }
  if (permC) {
    Ten t = C;
    t.p = pc;
    const std::string o = m + n + zs;
    for (size_t d = 0; d < o.size(); ++d) t.lens[d] = len[(unsigned char)o[d]];
    assign(ctx, 1.0, t, o.c_str(), beta, C, (sc + zs).c_str());
  }
}

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
  const std::string fa(ia), fb(ib), fc(ic);
  // a batch index (in A, B and C) must be the last index of all three: the
  // contraction then runs once per batch entry, as one batched GEMM
  char z = 0;
  if (!fa.empty() && fa.back() == fb.back() && fa.back() == fc.back())
    z = fa.back();
  const std::string sa = z ? fa.substr(0, fa.size() - 1) : fa;
  const std::string sb = z ? fb.substr(0, fb.size() - 1) : fb;
  const std::string sc = z ? fc.substr(0, fc.size() - 1) : fc;
  require((int)fa.size() == A.order && (int)fb.size() == B.order &&
              (int)fc.size() == C.order,
          "contract: index string / order mismatch: " + fa + "," + fb + "->" +
              fc);
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
  bind(fa, A);
  bind(fb, B);
  bind(fc, C);
  const int64_t nz = z ? len[(unsigned char)z] : 1;
  std::string M, N, K;
  for (char c : sa) {
    const bool inB = sb.find(c) != std::string::npos;
    const bool inC = sc.find(c) != std::string::npos;
    require(!(inB && inC), "contract: a batch index must be the last index of A, B and C");
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
  // emulated products with a constant operand (its panels cached) or an
  // operand or output to reorder (read or written in place where its indices
  // allow) take the panel route; its digits and products are those of the
  // plain route
  const bool emu_product = precision == GBCC_PREC_EMU && sK > 0 && sM > 1 && sN > 1 &&
                           2.0 * (double)sM * (double)sN * (double)sK >= ctx.emu_min_flops &&
                           nz < (1 << 20);
  const bool has_constant = ctx.use_panel_cache &&
                            (ctx.is_constant(A.p, sizeof(double) * A.size()) ||
                             ctx.is_constant(B.p, sizeof(double) * B.size()));
  if (emu_product && (has_constant || p.permA || p.permB || p.permC)) {
    contract_cached(ctx, alpha, A, sa, B, sb, beta, C, sc, p.m, p.n, p.k, p.permA, p.ta,
                    p.permB, p.tb, p.permC, p.swap, len, z, nz);
    return;
  }
  // operand A as a [M,K] (ta=0) or [K,M] (ta=1) matrix
  const double *pa = A.p;
  int64_t lda = p.ta ? sK : sM;
  DBuf ta_buf, tb_buf, tc_buf;
  if (p.permA) {
    ta_buf.alloc(ctx, sizeof(double) * A.size());
    Ten t = A;
    t.p = ta_buf.as<double>();
    const std::string o = p.m + p.k + (z ? std::string(1, z) : std::string());
    for (size_t d = 0; d < o.size(); ++d) t.lens[d] = len[(unsigned char)o[d]];
    assign(ctx, 1.0, A, fa.c_str(), 0.0, t, o.c_str());
    pa = t.p;
    lda = sM;
  }
  const double *pb = B.p;
  int64_t ldb = p.tb ? sN : sK;
  if (p.permB) {
    tb_buf.alloc(ctx, sizeof(double) * B.size());
    Ten t = B;
    t.p = tb_buf.as<double>();
    const std::string o = p.k + p.n + (z ? std::string(1, z) : std::string());
    for (size_t d = 0; d < o.size(); ++d) t.lens[d] = len[(unsigned char)o[d]];
    assign(ctx, 1.0, B, fb.c_str(), 0.0, t, o.c_str());
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
  // per-entry strides of a batched contraction
  const int64_t stA = sM * sK, stB = sK * sN, stC = sM * sN;
  if (!p.swap) {
    gemm(ctx, p.ta, p.tb, sM, sN, sK, alpha, pa, lda, pb, ldb, gbeta, pc, sM,
         nz, stA, stB, stC, precision);
  } else {
    // C^T[N,M] = op(B)^T op(A)^T
    gemm(ctx, !p.tb, !p.ta, sN, sM, sK, alpha, pb, ldb, pa, lda, gbeta, pc,
         sN, nz, stB, stA, stC, precision);
  }
  if (p.permC) {
    Ten t = C;
    t.p = pc;
    const std::string o = p.m + p.n + (z ? std::string(1, z) : std::string());
    for (size_t d = 0; d < o.size(); ++d) t.lens[d] = len[(unsigned char)o[d]];
    assign(ctx, 1.0, t, o.c_str(), beta, C, fc.c_str());
  }
}

}  // namespace gbcc
