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
  // tiled epilogue: rho_r = Permutation<3>(r); rinv[r][m] = rho_r^-1(m);
  // wpr[p][r] = spin/Fermi factor of sigma = rho_r o pi_p^-1
  int rinv[6][3];
  double wpr[6][6];
  double *DV;
  int ntile;            // tiles per dimension (16 wide)
};

constexpr int TT = 16;                 // epilogue tile edge
constexpr int TP = TT + 1;             // padded edge (odd strides: no bank conflicts)
constexpr int TILE_WORDS = TT * TP * TP;

__device__ __forceinline__ int tix(int i0, int i1, int i2) {
  return i0 + TP * (i1 + TP * i2);
}

// Pass 1: DV[abc] = (sum_p W_p[x_pi(0), x_pi(1), x_pi(2)]) / D_abc for one
// 16^3 tile, each permuted W_p tile staged through shared memory so that all
// global reads are coalesced (CcsdPerturbativeTriples.cxx:162-191).
__global__ void __launch_bounds__(256) triples_dv_kernel(EpiArgs a) {
  __shared__ double S[TILE_WORDS];
  const int64_t Nv = a.Nv;
  const int nt = a.ntile;
  int64_t b = blockIdx.x;
  const int tb[3] = {(int)(b % nt) * TT, (int)((b / nt) % nt) * TT, (int)(b / (nt * nt)) * TT};
  const int l0 = threadIdx.x % TT, l1 = threadIdx.x / TT;
  double acc[TT];
#pragma unroll
  for (int l2 = 0; l2 < TT; ++l2) acc[l2] = 0.0;
  for (int p = 0; p < 6; ++p) {
    const double *W = a.W[p];
    const int base0 = tb[a.dvp[p][0]], base1 = tb[a.dvp[p][1]], base2 = tb[a.dvp[p][2]];
    __syncthreads();
    for (int e = threadIdx.x; e < TT * TT * TT; e += blockDim.x) {
      const int i0 = e % TT, i1 = (e / TT) % TT, i2 = e / (TT * TT);
      const int64_t g0 = base0 + i0, g1 = base1 + i1, g2 = base2 + i2;
      S[tix(i0, i1, i2)] = (g0 < Nv && g1 < Nv && g2 < Nv) ? W[g0 + Nv * (g1 + Nv * g2)] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int l2 = 0; l2 < TT; ++l2) {
      const int x[3] = {l0, l1, l2};
      acc[l2] = __dadd_rn(acc[l2], S[tix(x[a.dvp[p][0]], x[a.dvp[p][1]], x[a.dvp[p][2]])]);
    }
  }
  const double ehs = __dadd_rn(__dadd_rn(a.eps_h[a.i3[0]], a.eps_h[a.i3[1]]), a.eps_h[a.i3[2]]);
  const int64_t ga = tb[0] + l0, gb = tb[1] + l1;
  if (ga >= Nv || gb >= Nv) return;
#pragma unroll
  for (int l2 = 0; l2 < TT; ++l2) {
    const int64_t gc = tb[2] + l2;
    if (gc >= Nv) break;
    double den = __dsub_rn(ehs, a.eps_p[ga]);
    den = __dsub_rn(den, a.eps_p[gb]);
    den = __dsub_rn(den, a.eps_p[gc]);
    a.DV[ga + Nv * (gb + Nv * gc)] = __ddiv_rn(acc[l2], den);
  }
}

// Pass 2: E += sum_{p distinct} sum_y X_p[y] sum_r wpr[p][r] DV[x_r(y)],
// x_r(y)_m = y_{rho_r^-1(m)}, X_p = W_p + S_p (the terms of
// CcsdPerturbativeTriples.cxx:193-214 regrouped so that each X_p is read once,
// in natural order); the six permuted DV tiles sit in shared memory.
__global__ void __launch_bounds__(256) triples_energy_kernel(EpiArgs a) {
  extern __shared__ double SD[];  // 6 tiles
  __shared__ double red[32];
  const int64_t Nv = a.Nv, No = a.No;
  const int nt = a.ntile;
  int64_t b = blockIdx.x;
  const int yb[3] = {(int)(b % nt) * TT, (int)((b / nt) % nt) * TT, (int)(b / (nt * nt)) * TT};
  for (int r = 0; r < 6; ++r) {
    double *T = SD + r * TILE_WORDS;
    const int base0 = yb[a.rinv[r][0]], base1 = yb[a.rinv[r][1]], base2 = yb[a.rinv[r][2]];
    for (int e = threadIdx.x; e < TT * TT * TT; e += blockDim.x) {
      const int i0 = e % TT, i1 = (e / TT) % TT, i2 = e / (TT * TT);
      const int64_t g0 = base0 + i0, g1 = base1 + i1, g2 = base2 + i2;
      T[tix(i0, i1, i2)] = (g0 < Nv && g1 < Nv && g2 < Nv) ? a.DV[g0 + Nv * (g1 + Nv * g2)] : 0.0;
    }
  }
  __syncthreads();
  const int l0 = threadIdx.x % TT, l1 = threadIdx.x / TT;
  const int64_t y0 = yb[0] + l0, y1 = yb[1] + l1;
  double acc = 0.0;
  if (y0 < Nv && y1 < Nv) {
    for (int l2 = 0; l2 < TT; ++l2) {
      const int64_t y2 = yb[2] + l2;
      if (y2 >= Nv) break;
      const int l[3] = {l0, l1, l2};
      double G[6];
#pragma unroll
      for (int r = 0; r < 6; ++r)
        G[r] = SD[r * TILE_WORDS + tix(l[a.rinv[r][0]], l[a.rinv[r][1]], l[a.rinv[r][2]])];
      const int64_t off = y0 + Nv * (y1 + Nv * y2);
#pragma unroll
      for (int p = 0; p < 6; ++p) {
        if (!a.distinct[p]) continue;
        const double sv = 0.5 * (a.T1[y0 + Nv * a.m[p][0]] *
                                 a.Vabij[y1 + Nv * (y2 + Nv * (a.m[p][1] + No * a.m[p][2]))]);
        const double x = a.W[p][off] + sv;
        double z = 0.0;
#pragma unroll
        for (int r = 0; r < 6; ++r) z = fma(a.wpr[p][r], G[r], z);
        acc = fma(x, z, acc);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  const int w = threadIdx.x / 32, ln = threadIdx.x % 32;
  if (ln == 0) red[w] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double r = (threadIdx.x < blockDim.x / 32) ? red[threadIdx.x] : 0.0;
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
  // tiled epilogue tables: rho_r^-1, and the factor of sigma = rho_r o pi_p^-1
  for (int r = 0; r < 6; ++r)
    for (int n = 0; n < 3; ++n) base.rinv[r][img[r][n]] = n;
  for (int p = 0; p < 6; ++p) {
    int pinv[3];
    for (int n = 0; n < 3; ++n) pinv[img[p][n]] = n;
    for (int r = 0; r < 6; ++r) {
      int inv = 0;
      for (int k = 0; k < 3; ++k) inv += (img[r][pinv[k]] == k);  // sigma(k) = rho(pi^-1(k))
      base.wpr[p][r] = spinf[inv];
    }
  }
  const int ntile = (int)((Nv + TT - 1) / TT);
  base.ntile = ntile;
  DBuf dvbuf(ctx, sizeof(double) * n3);
  base.DV = dvbuf.as<double>();
  const int epi_smem = 6 * TILE_WORDS * (int)sizeof(double);
  GBCC_CUDA(cudaFuncSetAttribute(triples_energy_kernel,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, epi_smem));
  int64_t ntrip = No * (No + 1) * (No + 2) / 6;
  const int nb = ntile * ntile * ntile;
  DBuf partials(ctx, sizeof(double) * nb * ntrip);
  DBuf per_trip(ctx, sizeof(double) * ntrip);
  // Precision mode: every operand family of the two W products is split into
  // digit panels once, so each W costs two tensor-core GEMM launches.
  //   Bw[z]   : Wvv[d,(b,c),z]   rows (b,c), K = d     (B role)
  //   At[x,y] : T2[a,d,x,y]      rows a,     K = d     (A role)
  //   Ah[x]   : T2[(a,b),x,l]    rows (a,b), K = l     (A role)
  //   Bh[y,z] : Vt[l,c,y,z]      rows c,     K = l     (B role)
  const bool emu = precision == GBCC_PREC_EMU;
  EmuPanels Bw, At, Ah, Bh;
  if (emu) {
    Bw = emu_split(ctx, false, Wvv.p(), Nv * Nv, Nv, Nv, 1, (int)No, n3);
    At = emu_split(ctx, true, T2, Nv, Nv, 1, Nv, (int)(No * No), Nv * Nv);
    Ah = emu_split(ctx, true, T2, Nv * Nv, No, 1, Nv * Nv * No, (int)No, Nv * Nv);
    Bh = emu_split(ctx, false, Vt.p(), Nv, No, No, 1, (int)(No * No), No * Nv);
    Wvv.buf.release();  // the FP64 copy is no longer needed
  }
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
          if (emu) {
            emu_gemm_panels(ctx, At, (int)(m[0] + No * m[1]), Bw, m[2], 1.0, 0.0, Wp, Nv);
            emu_gemm_panels(ctx, Ah, m[0], Bh, (int)(m[1] + No * m[2]), -1.0, 1.0, Wp,
                            Nv * Nv);
            continue;
          }
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
        triples_dv_kernel<<<nb, 256, 0, ctx.stream>>>(a);
        GBCC_CHECK_LAUNCH(ctx);
        triples_energy_kernel<<<nb, 256, epi_smem, ctx.stream>>>(a);
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
