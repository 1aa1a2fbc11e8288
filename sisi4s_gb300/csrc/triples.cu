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
//
// Precision mode: the two W products of every image are emulated-FP64 GEMMs
// on digit panels split once per (T) call.  The epilogue stays in FP64 in
// both modes: its terms cancel strongly, and rounding W or the epilogue
// arithmetic to FP32 moved E_(T) by ~1e-9 relative at No=32, Nv=256.  The FP64
// pipe of this GPU issues a few operations per clock per SM, so the epilogue
// is written to need few of them (cycle-type regrouping of the spin/Fermi
// weights, one division per element).

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
  const void *W[6];     // W_p (element type R) for each image p; aliases for repeats
  int distinct[6];
  int m[6][3];          // hole indices i o pi_p
  int img[6][3];        // Permutation<3>(s) images
  int dinv[6][3];       // D.V read: u_m = y_{dinv[p][m]}  (y_n = u_{pi_p(n)})
  int rinv[6][3];       // rho_r^-1: x_r(y)_m = y_{rinv[r][m]}
  int odd[6];           // parity of Permutation<3>(r)
  int i3[3];
  const double *eps_h;
  const void *eps_p, *T1h, *Vabij;   // element type R; T1h = T1 / 2
  int64_t Nv, No;
  const int *orbits;    // [norb][3] tile coordinates A <= B <= C
  double *partials;     // one per orbit
};

constexpr int OT = 8;                  // orbit tile edge
constexpr int OP = OT + 1;             // padded edge (odd strides: no bank conflicts)
constexpr int OT_WORDS = OT * OP * OP;
constexpr int OT_ELEMS = OT * OT * OT;
constexpr int EPI_THREADS = 256;
constexpr int EPI_PER = OT_ELEMS / EPI_THREADS;

__device__ __forceinline__ int find_tile(const int (*tl)[3], int n, int c0, int c1, int c2) {
  int j = 0;
  for (; j < n - 1; ++j)
    if (tl[j][0] == c0 && tl[j][1] == c1 && tl[j][2] == c2) break;
  return j;
}

// per-thread sum of products (FMA chain)
template <typename R> struct ProductSum {
  R s = R(0);
  __device__ void add(R x, R z) { s = fma(x, z, s); }
  __device__ double value() const { return (double)s; }
};

// One CTA per orbit of 8^3 tiles under the six coordinate permutations.
// Every permuted read of the triple's epilogue stays inside the orbit:
//   DV[u]  = (sum_p W_p[u_{pi_p(0)}, u_{pi_p(1)}, u_{pi_p(2)}]) / D_u
//            (CcsdPerturbativeTriples.cxx:162-191; p in Permutation<3> order)
//   E     += sum_{p distinct} sum_y X_p[y] Z_p[y],  X_p = W_p + S_p
//            (:193-214 regrouped so that X_p is read in natural order)
// with Z_p[y] = sum_r f(rho_r pi_p^-1) DV[x_r(y)].  The spin/Fermi factor f
// depends only on the cycle type: 8 for the identity (r = p), -4 for a
// transposition (r of the other parity), 2 for a 3-cycle, so
//   Z_p = 6 G_p + 2 G_same(p) - 4 G_other(p),   G_r = DV[x_r(y)],
// where G_even / G_odd sum G_r over even / odd r: two FMAs per (p, y).
// DV lives only in shared memory.  W_p tiles are read in natural order
// (coalesced) and scattered into the permuted D.V positions; for a fixed p
// the scatter is a bijection of the orbit onto itself.  R is the arithmetic
// type (double).
template <typename R>
__global__ void __launch_bounds__(EPI_THREADS, 3) triples_orbit_kernel(EpiArgs a) {
  __shared__ R DV[6 * OT_WORDS];
  __shared__ double red[EPI_THREADS / 32];
  const int64_t Nv = a.Nv, No = a.No;
  const R *__restrict__ eps_p = static_cast<const R *>(a.eps_p);
  const R *__restrict__ T1h = static_cast<const R *>(a.T1h);
  const R *__restrict__ Vabij = static_cast<const R *>(a.Vabij);
  const int rep[3] = {a.orbits[3 * blockIdx.x], a.orbits[3 * blockIdx.x + 1],
                      a.orbits[3 * blockIdx.x + 2]};
  int tl[6][3];
  int n = 0;
  for (int s = 0; s < 6; ++s) {
    const int c0 = rep[a.img[s][0]], c1 = rep[a.img[s][1]], c2 = rep[a.img[s][2]];
    bool seen = false;
    for (int j = 0; j < n; ++j) seen |= (tl[j][0] == c0 && tl[j][1] == c1 && tl[j][2] == c2);
    if (!seen) { tl[n][0] = c0; tl[n][1] = c1; tl[n][2] = c2; ++n; }
  }
  for (int i = threadIdx.x; i < 6 * OT_WORDS; i += EPI_THREADS) DV[i] = R(0);
  __syncthreads();
  // pass 1: permuted sum of the six W_p
  for (int p = 0; p < 6; ++p) {
    const R *__restrict__ W = static_cast<const R *>(a.W[p]);
    const int d0 = a.dinv[p][0], d1 = a.dinv[p][1], d2 = a.dinv[p][2];
    R v[6][EPI_PER];
#pragma unroll
    for (int j = 0; j < 6; ++j)
#pragma unroll
      for (int h = 0; h < EPI_PER; ++h) {
        v[j][h] = R(0);
        if (j < n) {
          const int e = threadIdx.x + EPI_THREADS * h;
          const int64_t g0 = tl[j][0] * OT + e % OT, g1 = tl[j][1] * OT + (e / OT) % OT,
                        g2 = tl[j][2] * OT + e / (OT * OT);
          if (g0 < Nv && g1 < Nv && g2 < Nv) v[j][h] = W[g0 + Nv * (g1 + Nv * g2)];
        }
      }
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      if (j >= n) break;
      const int jt = find_tile(tl, n, tl[j][d0], tl[j][d1], tl[j][d2]);
#pragma unroll
      for (int h = 0; h < EPI_PER; ++h) {
        const int e = threadIdx.x + EPI_THREADS * h;
        const int z[3] = {e % OT, (e / OT) % OT, e / (OT * OT)};
        R &t = DV[jt * OT_WORDS + z[d0] + OP * (z[d1] + OP * z[d2])];
        t = t + v[j][h];
      }
    }
    __syncthreads();
  }
  const R ehs = (R)__dadd_rn(__dadd_rn(a.eps_h[a.i3[0]], a.eps_h[a.i3[1]]), a.eps_h[a.i3[2]]);
  for (int j = 0; j < n; ++j)
    for (int e = threadIdx.x; e < OT_ELEMS; e += EPI_THREADS) {
      const int u0 = e % OT, u1 = (e / OT) % OT, u2 = e / (OT * OT);
      const int64_t g0 = tl[j][0] * OT + u0, g1 = tl[j][1] * OT + u1, g2 = tl[j][2] * OT + u2;
      R &t = DV[j * OT_WORDS + u0 + OP * (u1 + OP * u2)];
      if (g0 < Nv && g1 < Nv && g2 < Nv) {
        R den = ehs - eps_p[g0];
        den = den - eps_p[g1];
        den = den - eps_p[g2];
        t = __ddiv_rn(t, den);
      } else {
        t = R(0);
      }
    }
  __syncthreads();
  // pass 2: contraction with the spin/Fermi-weighted permutations of DV
  ProductSum<R> acc;
  for (int j = 0; j < n; ++j) {
    int jr[6];
#pragma unroll
    for (int r = 0; r < 6; ++r)
      jr[r] = find_tile(tl, n, tl[j][a.rinv[r][0]], tl[j][a.rinv[r][1]], tl[j][a.rinv[r][2]]);
#pragma unroll
    for (int h = 0; h < EPI_PER; ++h) {
      const int e = threadIdx.x + EPI_THREADS * h;
      const int z[3] = {e % OT, (e / OT) % OT, e / (OT * OT)};
      const int64_t y0 = tl[j][0] * OT + z[0], y1 = tl[j][1] * OT + z[1], y2 = tl[j][2] * OT + z[2];
      if (y0 >= Nv || y1 >= Nv || y2 >= Nv) continue;
      const int64_t off = y0 + Nv * (y1 + Nv * y2);
      R w[6];
#pragma unroll
      for (int p = 0; p < 6; ++p)
        w[p] = a.distinct[p] ? static_cast<const R *>(a.W[p])[off] : R(0);
      R G[6], ge = R(0), go = R(0);
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        G[r] = DV[jr[r] * OT_WORDS + z[a.rinv[r][0]] + OP * (z[a.rinv[r][1]] + OP * z[a.rinv[r][2]])];
        if (a.odd[r]) go = go + G[r];
        else ge = ge + G[r];
      }
      const R ze = R(2) * ge - R(4) * go, zo = R(2) * go - R(4) * ge;
#pragma unroll
      for (int p = 0; p < 6; ++p) {
        if (!a.distinct[p]) continue;
        const R x = fma(T1h[y0 + Nv * a.m[p][0]],
                        Vabij[y1 + Nv * (y2 + Nv * (a.m[p][1] + No * a.m[p][2]))], w[p]);
        const R zz = fma(R(6), G[p], a.odd[p] ? zo : ze);
        acc.add(x, zz);
      }
    }
  }
  double sum = acc.value();
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
  const int wi = threadIdx.x / 32, ln = threadIdx.x % 32;
  if (ln == 0) red[wi] = sum;
  __syncthreads();
  if (threadIdx.x < 32) {
    double r = (threadIdx.x < EPI_THREADS / 32) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    if (threadIdx.x == 0) a.partials[blockIdx.x] = r;
  }
}

// dst[i] = (R)(scale * src[i])
template <typename R>
__global__ void scaled_copy_kernel(const double *__restrict__ src, int64_t n, double scale,
                                   R *__restrict__ dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (R)(scale * src[i]);
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
  const int64_t No = I.No, Nv = I.Nv;
  const bool emu = precision == GBCC_PREC_EMU;
  using R = double;  // epilogue arithmetic type
  // Wvv[d,b,c,k] = sum_F Gab[F,b,d] Gai[F,c,k]
  OTen Wvv(ctx, {Nv, Nv, Nv, No});
  contract(ctx, 1.0, I.Gab, "Fbd", I.Gai, "Fck", 0.0, Wvv, "dbck", precision);
  // Vt[l,c,j,k] = Vijka[j,k,l,c]
  OTen Vt(ctx, {No, Nv, No, No});
  assign(ctx, 1.0, I.Vijka, "jklc", 0.0, Vt, "lcjk");
  const int64_t n3 = Nv * Nv * Nv;
  std::vector<DBuf> Wb(6);
  for (auto &b : Wb) b.alloc(ctx, sizeof(R) * n3);
  // T1 / 2 (exact scaling)
  DBuf t1h(ctx, sizeof(R) * Nv * No);
  scaled_copy_kernel<R><<<(unsigned)((Nv * No + 255) / 256), 256, 0, ctx.stream>>>(
      T1, Nv * No, 0.5, t1h.as<R>());
  GBCC_CHECK_LAUNCH(ctx);
  int img[6][3];
  for (int p = 0; p < 6; ++p) perm3(p, img[p]);
  EpiArgs base{};
  for (int p = 0; p < 6; ++p) {
    int inversions = 0;
    for (int n = 0; n < 3; ++n) {
      base.img[p][n] = img[p][n];
      base.dinv[p][img[p][n]] = n;
      base.rinv[p][img[p][n]] = n;
      for (int k = n + 1; k < 3; ++k) inversions += img[p][n] > img[p][k];
    }
    base.odd[p] = inversions & 1;
  }
  base.eps_h = I.eps_h.p();
  base.eps_p = I.eps_p.p();
  base.T1h = t1h.as<void>();
  base.Vabij = I.Vabij.p();
  base.Nv = Nv;
  base.No = No;
  // orbit representatives A <= B <= C of the 8^3 tiles
  const int ntile = (int)((Nv + OT - 1) / OT);
  std::vector<int> orb;
  for (int A = 0; A < ntile; ++A)
    for (int B = A; B < ntile; ++B)
      for (int Cc = B; Cc < ntile; ++Cc) {
        orb.push_back(A);
        orb.push_back(B);
        orb.push_back(Cc);
      }
  const int nb = (int)(orb.size() / 3);
  DBuf orbits(ctx, sizeof(int) * orb.size());
  GBCC_CUDA(cudaMemcpyAsync(orbits.as<int>(), orb.data(), sizeof(int) * orb.size(),
                            cudaMemcpyHostToDevice, ctx.stream));
  base.orbits = orbits.as<int>();
  int64_t ntrip = No * (No + 1) * (No + 2) / 6;
  DBuf partials(ctx, sizeof(double) * nb * ntrip);
  DBuf per_trip(ctx, sizeof(double) * ntrip);
  // Precision mode: every operand family of the two W products is split into
  // digit panels once, so each W costs two tensor-core GEMM launches.
  //   Bw[z]   : Wvv[d,(b,c),z]   rows (b,c), K = d     (B role)
  //   At[x,y] : T2[a,d,x,y]      rows a,     K = d     (A role)
  //   Ah[x]   : T2[(a,b),x,l]    rows (a,b), K = l     (A role)
  //   Bh[y,z] : Vt[l,c,y,z]      rows c,     K = l     (B role)
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
          a.W[p] = Wb[p].as<void>();
          double *Wp = Wb[p].as<double>();
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
        triples_orbit_kernel<R><<<nb, EPI_THREADS, 0, ctx.stream>>>(a);
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
