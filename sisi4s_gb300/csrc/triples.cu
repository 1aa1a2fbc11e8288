// Closed-shell (T) on the GPU.
//
// Follows CcsdPerturbativeTriples::run (src/algorithms/CcsdPerturbativeTriples.cxx:119-248):
// all 0 <= i <= j <= k < No; for each of the six Permutation<3> images pi of
// (i,j,k) that is distinct, the doubles contribution
//   W^{m}_{abc} = sum_d T_ad^{m0 m1} Wvv_{dbc}^{m2} - sum_l T_ab^{m0 l} V_{m1 m2 l c}
// (getDoublesContribution :88-96).  Unlike the reference, which rebuilds
// sum_F Gamma_Fbd Gamma_Fck for every permutation of every triple, the
// particle term uses Wvv[d,b,c,k] = sum_F Gamma_Fbd Gamma_Fck built once
// (Nv^3 No doubles).  The permuted sum D.V, the denominator (:183-191), the
// spin/Fermi-weighted T_abc (:193-212) and the energy contraction (:214) are
// one fused epilogue kernel per triple with a deterministic reduction.
#include <algorithm>
#include <vector>

#include "ccsd.hpp"

namespace gbcc {
namespace {

// Permutation<3>(p) images (src/math/Permutation.hpp:52-62)
void perm3(int p, int img[3]) {
  int sub[2];
  // Permutation<2>(p/3): p/3 even -> (0,1), odd -> (1,0)
  const int q = p / 3;
  if (q % 2 == 0) { sub[0] = 0; sub[1] = 1; } else { sub[0] = 1; sub[1] = 0; }
  const int r = p % 3;
  int i = 0;
  for (; i < r; ++i) img[i] = sub[i] + 1;
  img[r] = 0;
  for (++i; i < 3; ++i) img[i] = sub[i - 1] + 1;
}

struct EpiArgs {
  const double *W[6];
  int distinct[6];
  int m[6][3];          // hole indices i o pi_p
  int dvp[6][3];        // position n of the D.V read takes letter pi_p(n)
  int tp[6][6][3];      // [p][sigma][n] = sigma(pi_p(n))
  double sf[6];         // spin/Fermi factor of sigma
  int i3[3];
  const double *eps_h, *eps_p, *T1, *Vabij;
  int64_t Nv, No;
  double *partials;
};

__global__ void triples_epilogue_kernel(EpiArgs a) {
  __shared__ double sm[32];
  const int64_t Nv = a.Nv, No = a.No;
  const int64_t n3 = Nv * Nv * Nv;
  const double ehs = __dadd_rn(__dadd_rn(a.eps_h[a.i3[0]], a.eps_h[a.i3[1]]),
                               a.eps_h[a.i3[2]]);
  double acc = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n3;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t x[3];
    x[0] = e % Nv;
    x[1] = (e / Nv) % Nv;
    x[2] = e / (Nv * Nv);
    double dv = 0.0;
#pragma unroll
    for (int p = 0; p < 6; ++p) {
      const int64_t off = x[a.dvp[p][0]] + Nv * (x[a.dvp[p][1]] + Nv * x[a.dvp[p][2]]);
      dv = __dadd_rn(dv, a.W[p][off]);
    }
    double den = __dsub_rn(ehs, a.eps_p[x[0]]);
    den = __dsub_rn(den, a.eps_p[x[1]]);
    den = __dsub_rn(den, a.eps_p[x[2]]);
    dv = __ddiv_rn(dv, den);
    double t = 0.0;
#pragma unroll
    for (int p = 0; p < 6; ++p) {
      if (!a.distinct[p]) continue;
      const double *Wp = a.W[p];
      const int m0 = a.m[p][0], m1 = a.m[p][1], m2 = a.m[p][2];
      const double *t1 = a.T1 + Nv * m0;
      const double *vv = a.Vabij + Nv * Nv * (m1 + No * m2);
#pragma unroll
      for (int s = 0; s < 6; ++s) {
        const int64_t y0 = x[a.tp[p][s][0]], y1 = x[a.tp[p][s][1]],
                      y2 = x[a.tp[p][s][2]];
        const double w = Wp[y0 + Nv * (y1 + Nv * y2)];
        const double sv = 0.5 * (t1[y0] * vv[y1 + Nv * y2]);
        t = fma(a.sf[s], w + sv, t);
      }
    }
    acc = fma(dv, t, acc);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  if (l == 0) sm[w] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double r = (threadIdx.x < blockDim.x / 32) ? sm[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    if (threadIdx.x == 0) a.partials[blockIdx.x] = r;
  }
}

// out[t] = sum of partials[t][0..nb) ; one block per triple slot
__global__ void sum_rows_kernel(const double *__restrict__ partials, int nb,
                                double *__restrict__ out) {
  __shared__ double sm[32];
  double v = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) v += partials[(int64_t)blockIdx.x * nb + b];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  if (l == 0) sm[w] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double r = (threadIdx.x < blockDim.x / 32) ? sm[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    if (threadIdx.x == 0) out[blockIdx.x] = r;
  }
}

}  // namespace

// E_(T) for device-resident inputs.
double triples_energy(Context &ctx, const CcsdInputs &I, const double *T1,
                      const double *T2, int precision) {
  const int64_t No = I.No, Nv = I.Nv, NG = I.NG;
  const Ten T2t = ten(const_cast<double *>(T2), {Nv, Nv, No, No});
  (void)T2t;
  // Wvv[d,b,c,k] = sum_F Gab[F,b,d] Gai[F,c,k]
  OTen Wvv(ctx, {Nv, Nv, Nv, No});
  contract(ctx, 1.0, I.Gab, "Fbd", I.Gai, "Fck", 0.0, Wvv, "dbck", precision);
  (void)NG;
  // Vt[l,c,j,k] = Vijka[j,k,l,c]
  OTen Vt(ctx, {No, Nv, No, No});
  assign(ctx, 1.0, I.Vijka, "jklc", 0.0, Vt, "lcjk");
  const int64_t n3 = Nv * Nv * Nv;
  std::vector<DBuf> Wb(6);
  for (auto &b : Wb) b.alloc(ctx, sizeof(double) * n3);
  int img[6][3];
  for (int p = 0; p < 6; ++p) perm3(p, img[p]);
  EpiArgs base{};
  for (int p = 0; p < 6; ++p)
    for (int n = 0; n < 3; ++n) base.dvp[p][n] = img[p][n];
  for (int p = 0; p < 6; ++p)
    for (int s = 0; s < 6; ++s)
      for (int n = 0; n < 3; ++n) base.tp[p][s][n] = img[s][img[p][n]];
  const double spinf[4] = {2.0, -4.0, 0.0, 8.0};  // CcsdPerturbativeTriples.cxx:143
  for (int s = 0; s < 6; ++s) {
    int inv = 0;
    for (int n = 0; n < 3; ++n) inv += (img[s][n] == n);
    base.sf[s] = spinf[inv];
  }
  base.eps_h = I.eps_h.p();
  base.eps_p = I.eps_p.p();
  base.T1 = T1;
  base.Vabij = I.Vabij.p();
  base.Nv = Nv;
  base.No = No;
  int64_t ntrip = No * (No + 1) * (No + 2) / 6;
  int nb = (int)std::min<int64_t>((n3 + 255) / 256, (int64_t)std::max(ctx.sm_count, 1) * 4);
  DBuf partials(ctx, sizeof(double) * nb * ntrip);
  DBuf per_trip(ctx, sizeof(double) * ntrip);
  int64_t t = 0;
  for (int i0 = 0; i0 < No; ++i0)
    for (int i1 = i0; i1 < No; ++i1)
      for (int i2 = i1; i2 < No; ++i2, ++t) {
        const int iv[3] = {i0, i1, i2};
        EpiArgs a = base;
        a.i3[0] = i0; a.i3[1] = i1; a.i3[2] = i2;
        for (int p = 0; p < 6; ++p) {
          int m[3];
          for (int n = 0; n < 3; ++n) m[n] = iv[img[p][n]];
          int q = 0;
          for (; q < p; ++q)
            if (a.m[q][0] == m[0] && a.m[q][1] == m[1] && a.m[q][2] == m[2]) break;
          for (int n = 0; n < 3; ++n) a.m[p][n] = m[n];
          if (q < p) {                                            // :166-172
            a.distinct[p] = 0;
            a.W[p] = a.W[q];
            continue;
          }
          a.distinct[p] = 1;
          double *Wp = Wb[p].as<double>();
          a.W[p] = Wp;
          // W[a,(b,c)] = sum_d T2[a,d,m0,m1] Wvv[d,(b,c),m2]
          gemm(ctx, false, false, Nv, Nv * Nv, Nv, 1.0,
               T2 + Nv * Nv * (m[0] + No * m[1]), Nv, Wvv.p() + n3 * m[2], Nv,
               0.0, Wp, Nv, 1, 0, 0, 0, precision);
          // W[(a,b),c] -= sum_l T2[a,b,m0,l] Vt[l,c,m1,m2]
          gemm(ctx, false, false, Nv * Nv, Nv, No, -1.0,
               T2 + Nv * Nv * m[0], Nv * Nv * No,
               Vt.p() + No * Nv * (m[1] + No * m[2]), No, 1.0, Wp, Nv * Nv, 1,
               0, 0, 0, precision);
        }
        a.partials = partials.as<double>() + (int64_t)nb * t;
        triples_epilogue_kernel<<<nb, 256, 0, ctx.stream>>>(a);
        GBCC_CHECK_LAUNCH(ctx);
      }
  sum_rows_kernel<<<(unsigned)ntrip, 256, 0, ctx.stream>>>(partials.as<double>(), nb,
                                                           per_trip.as<double>());
  GBCC_CHECK_LAUNCH(ctx);
  std::vector<double> h(ntrip);
  GBCC_CUDA(cudaMemcpyAsync(h.data(), per_trip.as<double>(), 8 * ntrip,
                            cudaMemcpyDeviceToHost, ctx.stream));
  ctx.check_device_errors();
  double e = 0.0;
  for (double v : h) e += v;  // fixed (triple) order
  return e;
}

}  // namespace gbcc
