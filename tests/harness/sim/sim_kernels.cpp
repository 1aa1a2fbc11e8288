// Host models of libgbcc's kernel launchers (see sim.hpp).  Each follows the
// arithmetic of its kernel in ccsd_kernels.cu, tensor_ops.cu, gemm_f64.cu,
// gemm_emu.cu, triples.cu or ccsd_complex_kernels.cu, in FP64, and runs
// through sim::submit so that it is recorded while its stream is captured.
// Arrays that a launcher passes by value to its kernel (pointer lists, slot
// numbers) are copied into the recorded work here too.
#include <algorithm>
#include <array>
#include <cmath>
#include <vector>

#include "ccsd.hpp"
#include "ccsd_kernels.hpp"
#include "sim.hpp"

namespace gbcc {

// declared in device_backend.hpp
void conj_over_denominator(Context &ctx, double *re, double *im, const double *eh,
                           const double *ep, int64_t i0, int64_t i1, int64_t i2,
                           int64_t Nv);

namespace {

void launch(Context &ctx, sim::Op op) {
  ctx.launches++;
  sim::submit(ctx.stream, std::move(op));
}

// Permutation<3>(p) images, p = 0..5
const int kPerm[6][3] = {{0, 1, 2}, {1, 0, 2}, {1, 2, 0}, {0, 2, 1}, {2, 0, 1}, {2, 1, 0}};

}  // namespace

int reduction_blocks(const Context &ctx, int64_t n) {
  const int RT = 256;
  int64_t g = (n + RT * 4 - 1) / (RT * 4);
  const int64_t cap = (int64_t)(ctx.sm_count > 0 ? ctx.sm_count : 148) * 4;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

// ------------------------------------------------------------ tensor_ops.cu
void fill(Context &ctx, double *p, int64_t n, double v) {
  if (n <= 0) return;
  launch(ctx, [=]() { std::fill(p, p + n, v); });
}

void copy(Context &ctx, double *dst, const double *src, int64_t n) {
  if (n <= 0 || dst == src) return;
  GBCC_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                            ctx.stream));
}

void axpby(Context &ctx, int64_t n, double a, const double *x, double b, double *y) {
  if (n <= 0) return;
  launch(ctx, [=]() {
    for (int64_t i = 0; i < n; ++i) {
      double v = (a == 0.0) ? 0.0 : a * x[i];
      if (b != 0.0) v = v + b * y[i];
      y[i] = v;
    }
  });
}

void permute(Context &ctx, const Ten &src, const int *perm, double alpha, double beta,
             Ten &dst) {
  const int n = src.order;
  require(dst.order == n && n >= 1 && n <= 6, "permute: order mismatch");
  require(src.p != dst.p, "permute: in-place permutation is not supported");
  for (int q = 0; q < n; ++q)
    require(dst.lens[q] == src.lens[perm[q]], "permute: length mismatch");
  if (src.size() == 0) return;
  std::array<int64_t, 6> sstride{};
  int64_t s = 1;
  for (int q = 0; q < n; ++q) {
    sstride[q] = s;
    s *= src.lens[q];
  }
  std::array<int64_t, 6> map{};  // stride in src of each dst dimension
  for (int d = 0; d < n; ++d) map[d] = sstride[perm[d]];
  const Ten S = src, D = dst;
  launch(ctx, [=]() {
    const int64_t total = D.size();
    std::array<int64_t, 6> idx{};
    int64_t off = 0;
    for (int64_t e = 0; e < total; ++e) {
      double v = alpha * S.p[off];
      if (beta != 0.0) v = v + beta * D.p[e];
      D.p[e] = v;
      for (int d = 0; d < n; ++d) {  // next dst index, first index fastest
        ++idx[d];
        off += map[d];
        if (idx[d] < D.lens[d]) break;
        off -= map[d] * D.lens[d];
        idx[d] = 0;
      }
    }
  });
}

// --------------------------------------------------------------- gemm_*.cu
namespace {

void gemm_now(bool ta, bool tb, int64_t M, int64_t N, int64_t K, double alpha,
              const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
              double *C, int64_t ldc) {
  for (int64_t n = 0; n < N; ++n)
    for (int64_t m = 0; m < M; ++m) {
      double acc = 0.0;
      for (int64_t k = 0; k < K; ++k) {
        const double a = ta ? A[k + m * lda] : A[m + k * lda];
        const double b = tb ? B[n + k * ldb] : B[k + n * ldb];
        acc += a * b;
      }
      double v = alpha * acc;
      if (beta != 0.0) v += beta * C[m + n * ldc];
      C[m + n * ldc] = v;
    }
}

}  // namespace

void gemm(Context &ctx, bool ta, bool tb, int64_t M, int64_t N, int64_t K, double alpha,
          const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
          double *C, int64_t ldc, int64_t batch, int64_t sA, int64_t sB, int64_t sC,
          int precision) {
  (void)precision;
  if (M <= 0 || N <= 0) return;
  ctx.flops += 2.0 * (double)M * (double)N * (double)K * (double)batch;
  launch(ctx, [=]() {
    for (int64_t z = 0; z < batch; ++z)
      gemm_now(ta, tb, M, N, K, alpha, A + z * sA, lda, B + z * sB, ldb, beta, C + z * sC,
               ldc);
  });
}

// operand p, element (r, k) at base + p pstride + r rs + k ks, copied as
// panels[p][k][r]
EmuPanels emu_split(Context &ctx, bool role_a, const double *base, int64_t R, int64_t K,
                    int64_t rs, int64_t ks, int count, int64_t pstride, const IdxMap &map) {
  require(R > 0 && K > 0 && count > 0, "emu_split: empty operand");
  require((map.rl == 0 || R < (1LL << 31)) && (map.kl == 0 || K < (1LL << 31)),
          "emu_split: mapped dimension too large");
  EmuPanels P;
  P.role_a = role_a;
  P.S = ctx.emu_slices;
  P.rows = R;
  P.K = K;
  P.rs = rs;
  P.ks = ks;
  P.map = map;
  P.count = count;
  P.panels.alloc(ctx, sizeof(double) * (size_t)count * R * K);
  double *out = P.panels.as<double>();
  const IdxMap mp = map;
  auto off = [](int64_t v, int64_t s0, unsigned l, int64_t s1) {
    return l == 0 ? v * s0 : (v % l) * s0 + (v / l) * s1;
  };
  launch(ctx, [=]() {
    for (int p = 0; p < count; ++p)
      for (int64_t k = 0; k < K; ++k)
        for (int64_t r = 0; r < R; ++r)
          out[r + R * (k + K * p)] =
              base[p * pstride + off(r, rs, mp.rl, mp.rs1) + off(k, ks, mp.kl, mp.ks1)];
  });
  return P;
}

void emu_gemm_panels(Context &ctx, const EmuPanels &A, int ia, const EmuPanels &B, int ib,
                     double alpha, double beta, double *C, int64_t ldc, df32 *Cdf) {
  require(A.role_a && !B.role_a && A.K == B.K && A.S == B.S,
          "emu_gemm_panels: operand mismatch");
  require(ia >= 0 && ia < A.count && ib >= 0 && ib < B.count, "emu_gemm_panels: index");
  require(Cdf == nullptr, "simulation: float-float GEMM output is not modelled");
  const int64_t M = A.rows, N = B.rows, K = A.K;
  const double *a = A.panels.as<double>() + M * K * ia;
  const double *b = B.panels.as<double>() + N * K * ib;
  ctx.flops += 2.0 * (double)M * (double)N * (double)K;
  launch(ctx, [=]() {
    for (int64_t n = 0; n < N; ++n)
      for (int64_t m = 0; m < M; ++m) {
        double acc = 0.0;
        for (int64_t k = 0; k < K; ++k) acc += a[m + M * k] * b[n + N * k];
        double v = alpha * acc;
        if (beta != 0.0) v += beta * C[m + n * ldc];
        C[m + n * ldc] = v;
      }
  });
}

void emu_gemm_panels_mapped(Context &ctx, const EmuPanels &A, int ia, const EmuPanels &B,
                            int ib, double alpha, double beta, double *C, const OutMap &map) {
  require(A.role_a && !B.role_a && A.K == B.K && A.S == B.S,
          "emu_gemm_panels_mapped: operand mismatch");
  require(ia >= 0 && ia < A.count && ib >= 0 && ib < B.count, "emu_gemm_panels_mapped: index");
  require(map.ml0 > 0 && map.nl0 > 0, "emu_gemm_panels_mapped: empty map");
  const int64_t M = A.rows, N = B.rows, K = A.K;
  const double *a = A.panels.as<double>() + M * K * ia;
  const double *b = B.panels.as<double>() + N * K * ib;
  const OutMap mp = map;
  ctx.flops += 2.0 * (double)M * (double)N * (double)K;
  launch(ctx, [=]() {
    for (int64_t n = 0; n < N; ++n)
      for (int64_t m = 0; m < M; ++m) {
        double acc = 0.0;
        for (int64_t k = 0; k < K; ++k) acc += a[m + M * k] * b[n + N * k];
        double *q = C + (m % mp.ml0) * mp.ms0 + (m / mp.ml0) * mp.ms1 + (n % mp.nl0) * mp.ns0 +
                    (n / mp.nl0) * mp.ns1;
        double v = alpha * acc;
        if (beta != 0.0) v += beta * *q;
        *q = v;
      }
  });
}

void emu_gemm_panels_batched(Context &ctx, const EmuPanels &A, const EmuPanels &B, int nprob,
                             double alpha, double beta, double *C, int64_t ldc, int64_t sC,
                             const OutMap &map) {
  require(nprob >= 1 && nprob <= A.count && nprob <= B.count, "batched GEMM: operand count");
  for (int q = 0; q < nprob; ++q) {
    if (map.ml0 > 0) emu_gemm_panels_mapped(ctx, A, q, B, q, alpha, beta, C + (int64_t)q * sC, map);
    else emu_gemm_panels(ctx, A, q, B, q, alpha, beta, C + (int64_t)q * sC, ldc, nullptr);
  }
}

void gemm_emu_mapped(Context &ctx, bool ta, bool tb, int64_t M, int64_t N, int64_t K,
                     double alpha, const double *A, int64_t lda, const double *B, int64_t ldb,
                     double *C, const OutMap &map) {
  require(map.ml0 > 0 && map.nl0 > 0, "gemm_emu_mapped: empty map");
  const OutMap mp = map;
  ctx.flops += 2.0 * (double)M * (double)N * (double)K;
  launch(ctx, [=]() {
    for (int64_t n = 0; n < N; ++n)
      for (int64_t m = 0; m < M; ++m) {
        double acc = 0.0;
        for (int64_t k = 0; k < K; ++k) {
          const double a = ta ? A[k + m * lda] : A[m + k * lda];
          const double b = tb ? B[n + k * ldb] : B[k + n * ldb];
          acc += a * b;
        }
        C[(m % mp.ml0) * mp.ms0 + (m / mp.ml0) * mp.ms1 + (n % mp.nl0) * mp.ns0 +
          (n / mp.nl0) * mp.ns1] = alpha * acc;
      }
  });
}

EmuPanels emu_panels_alloc(Context &ctx, bool role_a, int64_t R, int64_t K) {
  require(R > 0 && K > 0, "emu_panels_alloc: empty operand");
  EmuPanels P;
  P.role_a = role_a;
  P.S = ctx.emu_slices;
  P.rows = R;
  P.K = K;
  P.count = 1;
  P.panels.alloc(ctx, sizeof(double) * (size_t)R * K);
  P.exps.alloc(ctx, sizeof(int) * (size_t)R);
  return P;
}

// the V product stored as the next product's operand, panels[k][r] with
// r = x + px y, k = d + pd c (m = x + px c, n = d + pd y), from operand
// panels (panels[p][k][r] as emu_split stores them)
void emu_gemm_panels_to_panels(Context &ctx, const EmuPanels &A, int ia, const EmuPanels &B,
                               int ib, int64_t px, int64_t pd, EmuPanels &P) {
  const int64_t M = A.rows, N = B.rows, K = A.K;
  require(A.role_a && !B.role_a && A.K == B.K && A.S == B.S && A.S == P.S,
          "emu_gemm_panels_to_panels: operand mismatch");
  require(ia >= 0 && ia < A.count && ib >= 0 && ib < B.count,
          "emu_gemm_panels_to_panels: index");
  require(P.role_a && P.count == 1, "emu_gemm_panels_to_panels: panels");
  require(px > 0 && pd > 0 && pd % 8 == 0 && M % px == 0 && N % pd == 0,
          "emu_gemm_panels_to_panels: shape");
  require(P.rows == px * (N / pd) && P.K == pd * (M / px),
          "emu_gemm_panels_to_panels: panel shape");
  ctx.flops += 2.0 * (double)M * (double)N * (double)K;
  const double *a = A.panels.as<double>() + M * K * ia;
  const double *b = B.panels.as<double>() + N * K * ib;
  double *out = P.panels.as<double>();
  const int64_t R = P.rows;
  launch(ctx, [=]() {
    for (int64_t n = 0; n < N; ++n)
      for (int64_t m = 0; m < M; ++m) {
        double acc = 0.0;
        for (int64_t k = 0; k < K; ++k) acc += a[m + M * k] * b[n + N * k];
        const int64_t x = m % px, c = m / px, d = n % pd, y = n / pd;
        out[(x + px * y) + R * (d + pd * c)] = acc;
      }
  });
}

// the bound kernels only set digit exponents, which the FP64 model ignores
void ladder_amax(Context &ctx, const double *dG, int64_t G, int64_t Nv, void *amax) {
  (void)dG; (void)G;
  double *a = static_cast<double *>(amax);
  launch(ctx, [=]() {
    for (int64_t i = 0; i < Nv; ++i) a[i] = 0.0;
  });
}

void ladder_row_exponents(Context &ctx, const void *amax, int64_t x0, int64_t nx, int64_t y0,
                          int64_t ny, int *er) {
  (void)amax; (void)x0; (void)y0;
  launch(ctx, [=]() {
    for (int64_t r = 0; r < nx * ny; ++r) er[r] = 0;
  });
}

void gemm_emu_noalloc(Context &ctx, bool ta, bool tb, int64_t M, int64_t N, int64_t K,
                      double alpha, const double *A, int64_t lda, const double *B,
                      int64_t ldb, double beta, double *C, int64_t ldc) {
  require(M > 0 && N > 0 && K > 0, "gbcc_dgemm_emu_noalloc: sizes must be positive");
  require(A && B && C, "gbcc_dgemm_emu_noalloc: null operand");
  gemm(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, 1, 0, 0, 0,
       GBCC_PREC_EMU);
}

// ---------------------------------------------------------- ccsd_kernels.cu
void outer_add(Context &ctx, double *X0, const double *T20, const double *T10, double c,
               int64_t Nv, int64_t No, int64_t nz) {
  const int64_t n2 = Nv * Nv * No * No;
  for (int64_t z = 0; z < nz; ++z)
  launch(ctx, [=]() {
    double *X = X0 + z * n2;
    const double *T2 = T20 + z * n2;
    const double *T1 = T10 + z * Nv * No;
    for (int64_t j = 0; j < No; ++j)
      for (int64_t i = 0; i < No; ++i)
        for (int64_t b = 0; b < Nv; ++b)
          for (int64_t a = 0; a < Nv; ++a) {
            const int64_t e = a + Nv * (b + Nv * (i + No * j));
            double p = T1[a + Nv * i] * T1[b + Nv * j];
            if (c != 1.0) p = c * p;
            X[e] = T2[e] + p;
          }
  });
}

void jacobi_update(Context &ctx, const FockLayout &L, const double *R, const double *T,
                   double *est, double *dT, const double *eps_h, const double *eps_p,
                   double shift, int nhist, const double *const *hist, double *partials,
                   double *sums) {
  require(nhist <= GBCC_MAX_DIIS, "too many DIIS vectors");
  (void)partials;
  const std::vector<const double *> h(hist, hist + nhist);
  const FockLayout F = L;
  launch(ctx, [=]() {
    std::vector<double> acc(2 + h.size(), 0.0);
    for (int64_t e = 0; e < F.ntot; ++e) {
      double d;
      if (e < F.n1) {
        d = eps_p[e % F.Nv] - eps_h[e / F.Nv];
      } else if (e >= F.off2 && e < F.off2 + F.n2) {
        int64_t r = e - F.off2;
        const int64_t a = r % F.Nv;
        r /= F.Nv;
        const int64_t b = r % F.Nv;
        r /= F.Nv;
        const int64_t i = r % F.No, j = r / F.No;
        d = ((eps_p[a] - eps_h[i]) + eps_p[b]) - eps_h[j];
      } else {
        est[e] = dT[e] = 0.0;
        continue;
      }
      const double t = T[e];
      double r = R[e];
      if (shift != 0.0) r = r - shift * t;
      const double es = -r / (d + shift);
      const double dt = es - t;
      est[e] = es;
      dT[e] = dt;
      acc[0] += dt * dt;
      acc[1] += es * es;
      for (size_t q = 0; q < h.size(); ++q) acc[2 + q] += dt * h[q][e];
    }
    std::copy(acc.begin(), acc.end(), sums);
  });
}

void energy_terms(Context &ctx, const double *T1, const double *T2, const double *V,
                  const double *Vx, int64_t Nv, int64_t No, double *partials,
                  double *sums4) {
  (void)partials;
  launch(ctx, [=]() {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int64_t n = Nv * Nv * No * No;
    for (int64_t e = 0; e < n; ++e) {
      int64_t r = e;
      const int64_t a = r % Nv;
      r /= Nv;
      const int64_t b = r % Nv;
      r /= Nv;
      const int64_t i = r % No, j = r / No;
      const double tt = T1[a + Nv * i] * T1[b + Nv * j];
      acc[0] += T2[e] * V[e];
      acc[1] += tt * V[e];
      acc[2] += T2[e] * Vx[e];
      acc[3] += tt * Vx[e];
    }
    std::copy(acc, acc + 4, sums4);
  });
}

void pair_energy(Context &ctx, const double *T1, const double *T2, const double *V,
                 const double *Vx, int64_t Nv, int64_t No, double *out) {
  launch(ctx, [=]() {
    for (int64_t j = 0; j < No; ++j)
      for (int64_t i = 0; i < No; ++i) {
        double s[4] = {0.0, 0.0, 0.0, 0.0};
        const int64_t base = Nv * Nv * (i + No * j);
        for (int64_t b = 0; b < Nv; ++b)
          for (int64_t a = 0; a < Nv; ++a) {
            const int64_t ab = a + Nv * b;
            const double tt = T1[a + Nv * i] * T1[b + Nv * j];
            s[0] += T2[base + ab] * V[base + ab];
            s[1] += T2[base + ab] * Vx[base + ab];
            s[2] += tt * V[base + ab];
            s[3] += tt * Vx[base + ab];
          }
        out[i + No * j] = 2.0 * s[0] + (-1.0) * s[1] + 2.0 * s[2] + (-1.0) * s[3];
      }
  });
}

void diis_solve(Context &ctx, double *B, int N, int k, int count, const double *sums,
                int nhist, const int *hist_slot, double *weights, double *lambda,
                int *status) {
  require(nhist <= GBCC_MAX_DIIS, "too many DIIS vectors");
  const std::vector<int> hs(hist_slot, hist_slot + nhist);
  launch(ctx, [=]() {
    const int ld = N + 1;
    B[(k + 1) + ld * (k + 1)] = 2.0 * sums[0];
    for (size_t q = 0; q < hs.size(); ++q) {
      const int i = hs[q];
      const double ov = 2.0 * sums[2 + q];
      B[(k + 1) + ld * (i + 1)] = ov;
      B[(i + 1) + ld * (k + 1)] = ov;
    }
    const int dim = count + 1;
    std::vector<double> M(dim * dim), x(dim);
    for (int c = 0; c < dim; ++c)
      for (int r = 0; r < dim; ++r) M[r + dim * c] = B[r + ld * c];
    for (int r = 0; r < dim; ++r) x[r] = (r == 0) ? -1.0 : 0.0;
    int st = 0;
    for (int c = 0; c < dim; ++c) {  // Gaussian elimination, partial pivoting
      int piv = c;
      double best = std::fabs(M[c + dim * c]);
      for (int r = c + 1; r < dim; ++r)
        if (std::fabs(M[r + dim * c]) > best) {
          best = std::fabs(M[r + dim * c]);
          piv = r;
        }
      if (!std::isfinite(best)) {  // overflowed overlaps
        st = 2;
        break;
      }
      if (!(best > 0.0)) {  // exact zero pivot
        st = 1;
        break;
      }
      if (piv != c) {
        for (int cc = 0; cc < dim; ++cc) std::swap(M[c + dim * cc], M[piv + dim * cc]);
        std::swap(x[c], x[piv]);
      }
      const double inv = 1.0 / M[c + dim * c];
      for (int r = c + 1; r < dim; ++r) {
        const double f = M[r + dim * c] * inv;
        if (f == 0.0) continue;
        for (int cc = c; cc < dim; ++cc) M[r + dim * cc] -= f * M[c + dim * cc];
        x[r] -= f * x[c];
      }
    }
    if (!st)
      for (int r = dim - 1; r >= 0; --r) {
        double s = x[r];
        for (int cc = r + 1; cc < dim; ++cc) s -= M[r + dim * cc] * x[cc];
        x[r] = s / M[r + dim * r];
        if (!std::isfinite(x[r])) st = 2;
      }
    *status = st;
    *lambda = st ? 0.0 : x[0];
    for (int j = 0; j < count; ++j) {
      const int i = (k + N - j) % N;
      weights[j] = st ? (j == 0 ? 1.0 : 0.0) : x[i + 1];
    }
  });
}

void diis_combine(Context &ctx, int count, const double *const *src, const double *w,
                  double *out, int64_t n, double *partials, double *sum) {
  (void)partials;
  const std::vector<const double *> s(src, src + count);
  launch(ctx, [=]() {
    double acc = 0.0;
    for (int64_t e = 0; e < n; ++e) {
      double v = 0.0;
      for (int j = 0; j < count; ++j) v = v + w[j] * s[j][e];
      out[e] = v;
      acc += v * v;
    }
    *sum = acc;
  });
}

void linear_mix(Context &ctx, double *next, double *nres, double *last, double *lres,
                double ratio, int64_t n, double *partials, double *sums2) {
  (void)partials;
  launch(ctx, [=]() {
    double a0 = 0.0, a1 = 0.0;
    const double q = 1.0 - ratio;
    for (int64_t e = 0; e < n; ++e) {
      const double l = last[e] * q;
      const double nx = next[e] * ratio + l;
      const double lr = lres[e] * q;
      const double nr = nres[e] * ratio + lr;
      last[e] = l;
      lres[e] = lr;
      next[e] = nx;
      nres[e] = nr;
      a0 += nr * nr;
      a1 += nx * nx;
    }
    sums2[0] = a0;
    sums2[1] = a1;
  });
}

void slice_add(Context &ctx, double *R0, const double *Rxy0, int64_t Nv, int64_t No,
               int64_t a0, int64_t b0, int64_t nx, int64_t ny, bool mirror, int64_t nz) {
  for (int64_t z = 0; z < nz; ++z)
  launch(ctx, [=]() {
    double *R = R0 + z * Nv * Nv * No * No;
    const double *Rxy = Rxy0 + z * nx * ny * No * No;
    for (int64_t j = 0; j < No; ++j)
      for (int64_t i = 0; i < No; ++i)
        for (int64_t y = 0; y < ny; ++y)
          for (int64_t x = 0; x < nx; ++x) {
            const double v = Rxy[x + nx * (y + ny * (i + No * j))];
            R[(a0 + x) + Nv * ((b0 + y) + Nv * (i + No * j))] += v;
            if (mirror) R[(b0 + y) + Nv * ((a0 + x) + Nv * (j + No * i))] += v;
          }
  });
}

void gather_slice(Context &ctx, double *dst0, const double *src0, int64_t G, int64_t Nv,
                  int64_t x0, int64_t nx, int64_t nz) {
  for (int64_t z = 0; z < nz; ++z)
  launch(ctx, [=]() {
    double *dst = dst0 + z * G * nx * Nv;
    const double *src = src0 + z * G * Nv * Nv;
    for (int64_t c = 0; c < Nv; ++c)
      for (int64_t x = 0; x < nx; ++x)
        for (int64_t g = 0; g < G; ++g)
          dst[g + G * (x + nx * c)] = src[g + G * ((x0 + x) + Nv * c)];
  });
}

void batch_gather(Context &ctx, const double *const *src_dev, int64_t n, int64_t nz,
                  double *dst) {
  launch(ctx, [=]() {
    for (int64_t z = 0; z < nz; ++z)
      for (int64_t e = 0; e < n; ++e) dst[z * n + e] = src_dev[z][e];
  });
}

void batch_scatter(Context &ctx, const double *src, int64_t n, int64_t nz,
                   double *const *dst_dev) {
  launch(ctx, [=]() {
    for (int64_t z = 0; z < nz; ++z)
      for (int64_t e = 0; e < n; ++e) dst_dev[z][e] = src[z * n + e];
  });
}

void vertex_block(Context &ctx, double *dst, const double *src, int64_t G, int64_t Np,
                  int64_t p0, int64_t np, int64_t q0, int64_t nq) {
  launch(ctx, [=]() {
    for (int64_t q = 0; q < nq; ++q)
      for (int64_t p = 0; p < np; ++p)
        for (int64_t g = 0; g < G; ++g)
          dst[g + G * (p + np * q)] = src[g + G * ((p0 + p) + Np * (q0 + q))];
  });
}

void any_nonzero(Context &ctx, const double *p, int64_t n, int *flag_dev) {
  GBCC_CUDA(cudaMemsetAsync(flag_dev, 0, sizeof(int), ctx.stream));
  launch(ctx, [=]() {
    for (int64_t e = 0; e < n; ++e)
      if (p[e] != 0.0) {
        *flag_dev = 1;
        return;
      }
  });
}

// --------------------------------------------------- ccsd_complex_kernels.cu
void conj_over_denominator(Context &ctx, double *re, double *im, const double *eh,
                           const double *ep, int64_t i0, int64_t i1, int64_t i2,
                           int64_t Nv) {
  launch(ctx, [=]() {
    const double hs = (eh[i0] + eh[i1]) + eh[i2];
    for (int64_t c = 0; c < Nv; ++c)
      for (int64_t b = 0; b < Nv; ++b)
        for (int64_t a = 0; a < Nv; ++a) {
          const int64_t e = a + Nv * (b + Nv * c);
          const double d = ((hs - ep[a]) - ep[b]) - ep[c];
          re[e] = re[e] / d;
          im[e] = -(im[e] / d);
        }
  });
}

// -------------------------------------------------------------- triples.cu
// Closed-shell (T) summed over all ordered (i, j, k) (the dense form of the
// reference loop, CcsdPerturbativeTriples.cxx:119-240):
//   W_abc^ijk = sum_d T_ad^ij Wvv_bdck - sum_l T_ab^il V_jklc,
//   Wvv_bdck = sum_G Gab_Gbd Gai_Gck,  S_abc^ijk = 1/2 T_a^i V_bc^jk,
//   E = sum (sum_pi W[pi] / D) (sum_sigma f(sigma) (W + S)[sigma abc]).
double triples_energy(Context &ctx, const CcsdInputs &I, const double *T1, const double *T2,
                      int precision) {
  (void)precision;
  require(I.Gab.p() && I.Gai.p() && I.Vabij.p() && I.Vijka.p(),
          "(T) needs the CoulombVertex");
  require(!sim::capturing(ctx.stream), "simulation: (T) inside a capture");
  const int64_t No = I.No, Nv = I.Nv, NG = I.NG;
  const double *Gab = I.Gab.p(), *Gai = I.Gai.p(), *V = I.Vabij.p(), *Vijka = I.Vijka.p();
  const double *eh = I.eps_h.p(), *ep = I.eps_p.p();
  std::vector<double> Wvv((size_t)(Nv * Nv * Nv * No), 0.0);  // [b,d,c,k]
  for (int64_t k = 0; k < No; ++k)
    for (int64_t c = 0; c < Nv; ++c)
      for (int64_t d = 0; d < Nv; ++d)
        for (int64_t b = 0; b < Nv; ++b) {
          double s = 0.0;
          for (int64_t g = 0; g < NG; ++g)
            s += Gab[g + NG * (b + Nv * d)] * Gai[g + NG * (c + Nv * k)];
          Wvv[b + Nv * (d + Nv * (c + Nv * k))] = s;
        }
  const int64_t n3 = Nv * Nv * Nv, o3 = No * No * No;
  std::vector<double> W((size_t)(n3 * o3)), X((size_t)(n3 * o3));
  auto at = [&](int64_t a, int64_t b, int64_t c, int64_t i, int64_t j, int64_t k) {
    return a + Nv * (b + Nv * (c + Nv * (i + No * (j + No * k))));
  };
  for (int64_t k = 0; k < No; ++k)
    for (int64_t j = 0; j < No; ++j)
      for (int64_t i = 0; i < No; ++i)
        for (int64_t c = 0; c < Nv; ++c)
          for (int64_t b = 0; b < Nv; ++b)
            for (int64_t a = 0; a < Nv; ++a) {
              double w = 0.0;
              for (int64_t d = 0; d < Nv; ++d)
                w += T2[a + Nv * (d + Nv * (i + No * j))] *
                     Wvv[b + Nv * (d + Nv * (c + Nv * k))];
              for (int64_t l = 0; l < No; ++l)
                w -= T2[a + Nv * (b + Nv * (i + No * l))] *
                     Vijka[j + No * (k + No * (l + No * c))];
              const int64_t e = at(a, b, c, i, j, k);
              W[e] = w;
              X[e] = w + 0.5 * T1[a + Nv * i] * V[b + Nv * (c + Nv * (j + No * k))];
            }
  const double sf[4] = {2.0, -4.0, 0.0, 8.0};  // by the number of fixed points
  double E = 0.0;
  for (int64_t k = 0; k < No; ++k)
    for (int64_t j = 0; j < No; ++j)
      for (int64_t i = 0; i < No; ++i)
        for (int64_t c = 0; c < Nv; ++c)
          for (int64_t b = 0; b < Nv; ++b)
            for (int64_t a = 0; a < Nv; ++a) {
              const int64_t v[3] = {a, b, c}, o[3] = {i, j, k};
              double dv = 0.0, z = 0.0;
              for (int p = 0; p < 6; ++p) {
                const int *q = kPerm[p];
                dv += W[at(v[q[0]], v[q[1]], v[q[2]], o[q[0]], o[q[1]], o[q[2]])];
                const int fixed = (q[0] == 0) + (q[1] == 1) + (q[2] == 2);
                z += sf[fixed] * X[at(v[q[0]], v[q[1]], v[q[2]], i, j, k)];
              }
              const double D = (((eh[i] + eh[j]) + eh[k]) - ep[a]) - ep[b] - ep[c];
              E += dv / D * z;
            }
  ctx.launches++;
  return E;
}

}  // namespace gbcc
