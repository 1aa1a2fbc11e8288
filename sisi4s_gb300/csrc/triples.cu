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
// on digit panels split once per (T) call, written as float-float pairs
// (hi + lo, ~48 bits) rounded from their exact fixed-point totals, and the
// epilogue computes in float-float.  Its terms cancel strongly: rounding W or
// the epilogue arithmetic to plain FP32 moved E_(T) by ~1e-9 relative at
// No=32, Nv=256, far above 1 uHa.  Float-float keeps FP64-level accuracy
// while running on the FP32 pipe; the FP64 pipe of this GPU issues a few
// operations per clock per SM, so an FP64 epilogue costs as much as the
// GEMMs.  FP64 mode runs the same kernel in double.

#include <algorithm>
#include <array>
#include <cmath>
#include <vector>

#include "ccsd.hpp"
#include "df32.hpp"

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

// what the epilogue needs of one hole triple (i <= j <= k)
struct EpiTriple {
  const void *W[6];     // W_p (element type R) for each image p; aliases for repeats
  int distinct[6];
  int m[6][3];          // hole indices i o pi_p
  int i3[3];
  int64_t t;            // index of the triple in the i <= j <= k order
};

struct EpiArgs {
  const EpiTriple *trip;  // one per blockIdx.y
  int img[6][3];        // Permutation<3>(s) images
  int dinv[6][3];       // D.V read: u_m = y_{dinv[p][m]}  (y_n = u_{pi_p(n)});
                        // also rho_r^-1 of the energy read, x_r(y)_m = y_{dinv[r][m]}
  int odd[6];           // parity of Permutation<3>(r)
  const double *eps_h;
  const void *eps_p, *T1h, *Vabij;   // element type R; T1h = T1 / 2
  int64_t Nv, No;
  const int *orbits;    // [norb][3] tile coordinates A <= B <= C
  double *partials;     // [triple][orbit]
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

// Arithmetic of the epilogue type R: double in FP64 mode, float-float
// (df32) in precision mode, where the FP32 pipe does the work.
__device__ __forceinline__ double ar_add(double a, double b) { return a + b; }
__device__ __forceinline__ double ar_sub(double a, double b) { return a - b; }
__device__ __forceinline__ double ar_madd(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ double ar_scale(double a, float k) { return (double)k * a; }
__device__ __forceinline__ double ar_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double ar_to_double(double a) { return a; }
__device__ __forceinline__ void ar_set(double &r, double x) { r = x; }
__device__ __forceinline__ df32 ar_add(df32 a, df32 b) { return df_add(a, b); }
__device__ __forceinline__ df32 ar_sub(df32 a, df32 b) { return df_sub(a, b); }
__device__ __forceinline__ df32 ar_madd(df32 a, df32 b, df32 c) { return df_add(df_mul(a, b), c); }
__device__ __forceinline__ df32 ar_scale(df32 a, float k) { return df_mulf(a, k); }
__device__ __forceinline__ df32 ar_div(df32 a, df32 b) { return df_div(a, b); }
__device__ __forceinline__ double ar_to_double(df32 a) { return df_to_double(a); }
__device__ __forceinline__ void ar_set(df32 &r, double x) { r = df_from_double(x); }

__device__ __forceinline__ double ar_shfl_down(double v, int o) {
  return __shfl_down_sync(0xffffffffu, v, o);
}
__device__ __forceinline__ df32 ar_shfl_down(df32 v, int o) {
  return df_make(__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o));
}

template <typename R>
__device__ __forceinline__ R ar_zero() {
  R r;
  ar_set(r, 0.0);
  return r;
}

// per-thread sum of products
template <typename R> struct ProductSum {
  R s = ar_zero<R>();
  __device__ void add(R x, R z) { s = ar_madd(x, z, s); }
  __device__ double value() const { return ar_to_double(s); }
};

// One CTA per orbit of 8^3 tiles under the six coordinate permutations
// (blockIdx.x) and per hole triple of the batch (blockIdx.y).
// Every permuted read of the triple's epilogue stays inside the orbit:
//   DV[u]  = (sum_p W_p[u_{pi_p(0)}, u_{pi_p(1)}, u_{pi_p(2)}]) / D_u
//            (CcsdPerturbativeTriples.cxx:162-191; p in Permutation<3> order)
//   E     += sum_{p distinct} sum_y X_p[y] Z_p[y],  X_p = W_p + S_p
//            (:193-214 regrouped so that X_p is read in natural order)
// with Z_p[y] = sum_r f(rho_r pi_p^-1) DV[x_r(y)].  The spin/Fermi factor f
// depends only on the cycle type: 8 for the identity (r = p), -4 for a
// transposition (r of the other parity), 2 for a 3-cycle, so
//   Z_p = 6 G_p + 2 G_same(p) - 4 G_other(p),   G_r = DV[x_r(y)],
// where G_even / G_odd sum G_r over even / odd r.
// DV lives only in shared memory.  W_p tiles are read in natural order
// (coalesced) and scattered into the permuted D.V positions; for a fixed p
// the scatter is a bijection of the orbit onto itself.  Both permuted
// shared-memory accesses (the scatter by pi_p and the read of x_r(y)) put
// local coordinate z_k at stride OP^img[p][k], and move tile j to the orbit
// tile jt[p][j]; these tables are built once per CTA.  R is the arithmetic
// type: double, or float-float in precision mode.
template <typename R>
__global__ void __launch_bounds__(EPI_THREADS, 4) triples_orbit_kernel(EpiArgs a) {
  __shared__ R DV[6 * OT_WORDS];
  __shared__ int s_jt[6][6];         // [p][j]: orbit tile of tile j moved by image p
  __shared__ int s_ps[6][3];         // [p][k]: shared-memory stride of z_k under image p
  __shared__ int s_org[6][3];        // first global coordinate of tile j
  __shared__ int s_lim[6][3];        // valid extent of tile j per dimension
  __shared__ int64_t s_gbase[6];     // global offset of the first element of tile j
  __shared__ const R *s_W[6];        // W_p
  __shared__ int64_t s_t1[6], s_v[6];  // offsets of T1h[:, m0] and Vabij[:, :, m1, m2]
  __shared__ int s_dist[6], s_odd[6], s_n;
  __shared__ R s_ehs;                // eps_i + eps_j + eps_k
  const int64_t Nv = a.Nv, No = a.No;
  const R *__restrict__ eps_p = static_cast<const R *>(a.eps_p);
  const R *__restrict__ T1h = static_cast<const R *>(a.T1h);
  const R *__restrict__ Vabij = static_cast<const R *>(a.Vabij);
  const EpiTriple &tr = a.trip[blockIdx.y];
  if (threadIdx.x == 0) {
    const int rep[3] = {a.orbits[3 * blockIdx.x], a.orbits[3 * blockIdx.x + 1],
                        a.orbits[3 * blockIdx.x + 2]};
    int tl[6][3];
    int n = 0;
    for (int q = 0; q < 6; ++q) {
      const int c0 = rep[a.img[q][0]], c1 = rep[a.img[q][1]], c2 = rep[a.img[q][2]];
      bool seen = false;
      for (int j = 0; j < n; ++j) seen |= (tl[j][0] == c0 && tl[j][1] == c1 && tl[j][2] == c2);
      if (!seen) { tl[n][0] = c0; tl[n][1] = c1; tl[n][2] = c2; ++n; }
    }
    for (int j = 0; j < n; ++j) {
      for (int k = 0; k < 3; ++k) {
        s_org[j][k] = tl[j][k] * OT;
        const int64_t rest = Nv - (int64_t)tl[j][k] * OT;
        s_lim[j][k] = rest < OT ? (int)rest : OT;
      }
      s_gbase[j] = s_org[j][0] + Nv * (s_org[j][1] + Nv * (int64_t)s_org[j][2]);
    }
    for (int q = 0; q < 6; ++q) {
      for (int k = 0; k < 3; ++k) s_ps[q][k] = a.img[q][k] == 0 ? 1 : (a.img[q][k] == 1 ? OP : OP * OP);
      for (int j = 0; j < n; ++j)
        s_jt[q][j] = find_tile(tl, n, tl[j][a.dinv[q][0]], tl[j][a.dinv[q][1]], tl[j][a.dinv[q][2]]);
      s_W[q] = static_cast<const R *>(tr.W[q]);
      s_t1[q] = Nv * tr.m[q][0];
      s_v[q] = Nv * Nv * (tr.m[q][1] + No * tr.m[q][2]);
      s_dist[q] = tr.distinct[q];
      s_odd[q] = a.odd[q];
    }
    s_n = n;
    ar_set(s_ehs, __dadd_rn(__dadd_rn(a.eps_h[tr.i3[0]], a.eps_h[tr.i3[1]]), a.eps_h[tr.i3[2]]));
  }
  for (int i = threadIdx.x; i < 6 * OT_WORDS; i += EPI_THREADS) DV[i] = ar_zero<R>();
  __syncthreads();
  const int n = s_n;
  // pass 1: permuted sum of the six W_p; this thread's local coordinates are
  // e = tid + 256 h, z0 fastest
#pragma unroll 1
  for (int p = 0; p < 6; ++p) {
    const R *__restrict__ W = s_W[p];
    R v[6][EPI_PER];
#pragma unroll
    for (int j = 0; j < 6; ++j)
#pragma unroll
      for (int h = 0; h < EPI_PER; ++h) {
        const int e = threadIdx.x + EPI_THREADS * h;
        const int z0 = e % OT, z1 = (e / OT) % OT, z2 = e / (OT * OT);
        v[j][h] = ar_zero<R>();
        if (j < n && z0 < s_lim[j][0] && z1 < s_lim[j][1] && z2 < s_lim[j][2])
          v[j][h] = W[s_gbase[j] + z0 + Nv * (z1 + Nv * z2)];
      }
    const int ps0 = s_ps[p][0], ps1 = s_ps[p][1], ps2 = s_ps[p][2];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      if (j >= n) break;
      const int base = s_jt[p][j] * OT_WORDS;
#pragma unroll
      for (int h = 0; h < EPI_PER; ++h) {
        const int e = threadIdx.x + EPI_THREADS * h;
        R &t = DV[base + (e % OT) * ps0 + ((e / OT) % OT) * ps1 + (e / (OT * OT)) * ps2];
        t = ar_add(t, v[j][h]);
      }
    }
    __syncthreads();
  }
  const R ehs = s_ehs;
  for (int j = 0; j < n; ++j)
#pragma unroll
    for (int h = 0; h < EPI_PER; ++h) {
      const int e = threadIdx.x + EPI_THREADS * h;
      const int z0 = e % OT, z1 = (e / OT) % OT, z2 = e / (OT * OT);
      R &t = DV[j * OT_WORDS + z0 + OP * (z1 + OP * z2)];
      if (z0 < s_lim[j][0] && z1 < s_lim[j][1] && z2 < s_lim[j][2]) {
        R den = ar_sub(ehs, eps_p[s_org[j][0] + z0]);
        den = ar_sub(den, eps_p[s_org[j][1] + z1]);
        den = ar_sub(den, eps_p[s_org[j][2] + z2]);
        t = ar_div(t, den);
      } else {
        t = ar_zero<R>();
      }
    }
  __syncthreads();
  // pass 2: contraction with the spin/Fermi-weighted permutations of DV
  ProductSum<R> acc;
#pragma unroll 1
  for (int jh = 0; jh < n * EPI_PER; ++jh) {
    const int j = jh / EPI_PER, e = threadIdx.x + EPI_THREADS * (jh % EPI_PER);
    const int z0 = e % OT, z1 = (e / OT) % OT, z2 = e / (OT * OT);
    if (z0 >= s_lim[j][0] || z1 >= s_lim[j][1] || z2 >= s_lim[j][2]) continue;
    const int64_t y0 = s_org[j][0] + z0;
    const int64_t y12 = (s_org[j][1] + z1) + Nv * (int64_t)(s_org[j][2] + z2);
    const int64_t off = s_gbase[j] + z0 + Nv * (z1 + Nv * z2);
    R G[6], ge = ar_zero<R>(), go = ar_zero<R>();
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      G[r] = DV[s_jt[r][j] * OT_WORDS + z0 * s_ps[r][0] + z1 * s_ps[r][1] + z2 * s_ps[r][2]];
      if (s_odd[r]) go = ar_add(go, G[r]);
      else ge = ar_add(ge, G[r]);
    }
    const R ze = ar_sub(ar_scale(ge, 2.0f), ar_scale(go, 4.0f));
    const R zo = ar_sub(ar_scale(go, 2.0f), ar_scale(ge, 4.0f));
#pragma unroll
    for (int p = 0; p < 6; ++p) {
      if (!s_dist[p]) continue;
      const R x = ar_madd(T1h[y0 + s_t1[p]], Vabij[y12 + s_v[p]], s_W[p][off]);
      const R zz = ar_add(ar_scale(G[p], 6.0f), s_odd[p] ? zo : ze);
      acc.add(x, zz);
    }
  }
  // block sum in the epilogue type; one conversion to double per CTA
  __shared__ R red[EPI_THREADS / 32];
  R sum = acc.s;
  for (int o = 16; o > 0; o >>= 1) sum = ar_add(sum, ar_shfl_down(sum, o));
  const int wi = threadIdx.x / 32, ln = threadIdx.x % 32;
  if (ln == 0) red[wi] = sum;
  __syncthreads();
  if (threadIdx.x < 32) {
    R r = (threadIdx.x < EPI_THREADS / 32) ? red[threadIdx.x] : ar_zero<R>();
    for (int o = 16; o > 0; o >>= 1) r = ar_add(r, ar_shfl_down(r, o));
    if (threadIdx.x == 0)
      a.partials[tr.t * (int64_t)gridDim.x + blockIdx.x] = ar_to_double(r);
  }
}

// dst[i] = scale * src[i] in the epilogue type (scale a power of two)
template <typename R>
__global__ void scaled_copy_kernel(const double *__restrict__ src, int64_t n, double scale,
                                   R *__restrict__ dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    ar_set(dst[i], scale * src[i]);
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
  // a solver of the stored formulation may have been set up without a vertex
  require(I.Gab.p() && I.Gai.p() && I.Vabij.p() && I.Vijka.p(),
          "(T) needs the CoulombVertex");
  const int64_t No = I.No, Nv = I.Nv;
  // Precision mode: W is produced as float-float by the emulated GEMMs and the
  // epilogue computes in float-float; FP64 mode computes in double.  Both
  // element types are 8 bytes.
  const bool emu = precision == GBCC_PREC_EMU;
  static_assert(sizeof(df32) == sizeof(double), "epilogue element size");
  // (T) in precision mode uses one more digit than the CCSD iteration: its
  // energy can be orders of magnitude larger than E_CCSD on far-from-converged
  // amplitudes (a chaotic DIIS trajectory), and it is the per-element
  // accuracy of W that its error follows
  struct SlicesScope {
    Context &c;
    int saved;
    ~SlicesScope() { c.emu_slices = saved; }
  } slices_scope{ctx, ctx.emu_slices};
  if (emu) ctx.emu_slices = std::min(8, ctx.emu_slices + 1);
  // Wvv[d,b,c,k] = sum_F Gab[F,b,d] Gai[F,c,k]
  OTen Wvv(ctx, {Nv, Nv, Nv, No});
  contract(ctx, 1.0, I.Gab, "Fbd", I.Gai, "Fck", 0.0, Wvv, "dbck", precision);
  // Vt[l,c,j,k] = Vijka[j,k,l,c]
  OTen Vt(ctx, {No, Nv, No, No});
  assign(ctx, 1.0, I.Vijka, "jklc", 0.0, Vt, "lcjk");
  const int64_t n3 = Nv * Nv * Nv;
  // epilogue operands in the epilogue type: T1 / 2 (exact scaling), and in
  // precision mode float-float copies of eps_p and Vabij
  const int64_t nv4 = Nv * Nv * No * No;
  auto convert = [&](const double *src, int64_t n, double scale, void *dst) {
    const unsigned g = (unsigned)std::min<int64_t>((n + 255) / 256, 8192);
    if (emu)
      scaled_copy_kernel<df32><<<g, 256, 0, ctx.stream>>>(src, n, scale, static_cast<df32 *>(dst));
    else
      scaled_copy_kernel<double><<<g, 256, 0, ctx.stream>>>(src, n, scale,
                                                            static_cast<double *>(dst));
    GBCC_CHECK_LAUNCH(ctx);
  };
  DBuf t1h(ctx, 8 * Nv * No), epsr, vr;
  convert(T1, Nv * No, 0.5, t1h.as<void>());
  if (emu) {
    epsr.alloc(ctx, 8 * Nv);
    vr.alloc(ctx, 8 * nv4);
    convert(I.eps_p.p(), Nv, 1.0, epsr.as<void>());
    convert(I.Vabij.p(), nv4, 1.0, vr.as<void>());
  }
  int img[6][3];
  for (int p = 0; p < 6; ++p) perm3(p, img[p]);
  EpiArgs base{};
  for (int p = 0; p < 6; ++p) {
    int inversions = 0;
    for (int n = 0; n < 3; ++n) {
      base.img[p][n] = img[p][n];
      base.dinv[p][img[p][n]] = n;
      for (int k = n + 1; k < 3; ++k) inversions += img[p][n] > img[p][k];
    }
    base.odd[p] = inversions & 1;
  }
  base.eps_h = I.eps_h.p();
  base.eps_p = emu ? epsr.as<void>() : static_cast<const void *>(I.eps_p.p());
  base.T1h = t1h.as<void>();
  base.Vabij = emu ? vr.as<void>() : static_cast<const void *>(I.Vabij.p());
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
  // Triples run in batches: the distinct images of a batch's triples get
  // their own W slots, so that all hole products of the batch are one grouped
  // tensor-core launch, all particle products another, and the epilogue one
  // launch over (orbit, triple).  The slot pool takes at most a quarter of
  // the free device memory (8 GiB at most, 6 slots at least) unless the
  // context sets the batch size.
  size_t free_b = 0, total_b = 0;
  GBCC_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const double slot_bytes = 8.0 * (double)n3;
  const int max_slots =
      ctx.triples_batch_images > 0
          ? std::max(6, ctx.triples_batch_images)
          : (int)std::max<double>(
                6.0, std::min(192.0, std::floor(std::min(free_b / 4.0, 8.0 * (1ull << 30)) /
                                                slot_bytes)));
  DBuf pool(ctx, (size_t)max_slots * 8 * (size_t)n3);
  auto slot_ptr = [&](int q) { return pool.as<double>() + (int64_t)q * n3; };
  std::vector<EpiTriple> trips;
  std::vector<int> h_ia, h_ib, p_ia, p_ib;     // hole / particle operand indices
  std::vector<df32 *> cdf;                     // output slot per problem
  std::vector<std::array<int, 3>> img_m;       // m per problem (FP64 mode)
  auto flush = [&]() {
    if (trips.empty()) return;
    const int np = (int)cdf.size();
    if (emu) {
      // the short-K hole products first (beta = 0: no read of W), then the
      // particle products accumulate, their C reads hidden behind K = Nv
      emu_gemm_panels_grouped(ctx, Ah, h_ia.data(), Bh, h_ib.data(), np, -1.0, 0.0,
                              nullptr, cdf.data(), Nv * Nv);
      emu_gemm_panels_grouped(ctx, At, p_ia.data(), Bw, p_ib.data(), np, 1.0, 1.0,
                              nullptr, cdf.data(), Nv);
    } else {
      for (int q = 0; q < np; ++q) {
        const int *m = img_m[q].data();
        double *Wp = slot_ptr(q);
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
    }
    DBuf tbuf(ctx, sizeof(EpiTriple) * trips.size());
    GBCC_CUDA(cudaMemcpyAsync(tbuf.as<EpiTriple>(), trips.data(),
                              sizeof(EpiTriple) * trips.size(), cudaMemcpyHostToDevice,
                              ctx.stream));
    EpiArgs a = base;
    a.trip = tbuf.as<EpiTriple>();
    a.partials = partials.as<double>();
    const dim3 grid((unsigned)nb, (unsigned)trips.size());
    if (emu)
      triples_orbit_kernel<df32><<<grid, EPI_THREADS, 0, ctx.stream>>>(a);
    else
      triples_orbit_kernel<double><<<grid, EPI_THREADS, 0, ctx.stream>>>(a);
    GBCC_CHECK_LAUNCH(ctx);
    trips.clear();
    h_ia.clear(); h_ib.clear(); p_ia.clear(); p_ib.clear();
    cdf.clear(); img_m.clear();
  };
  int64_t t = 0;
  for (int i0 = 0; i0 < No; ++i0)
    for (int i1 = i0; i1 < No; ++i1)
      for (int i2 = i1; i2 < No; ++i2, ++t) {
        const int iv[3] = {i0, i1, i2};
        const int ndist = (i0 == i1 && i1 == i2) ? 1 : ((i0 == i1 || i1 == i2) ? 3 : 6);
        if ((int)cdf.size() + ndist > max_slots || trips.size() >= 65535) flush();
        EpiTriple tr{};
        tr.i3[0] = i0; tr.i3[1] = i1; tr.i3[2] = i2;
        tr.t = t;
        for (int p = 0; p < 6; ++p) {
          int m[3];
          for (int n = 0; n < 3; ++n) m[n] = iv[img[p][n]];
          int q = 0;
          for (; q < p; ++q)
            if (tr.m[q][0] == m[0] && tr.m[q][1] == m[1] && tr.m[q][2] == m[2]) break;
          for (int n = 0; n < 3; ++n) tr.m[p][n] = m[n];
          if (q < p) {                                            // :166-172
            tr.distinct[p] = 0;
            tr.W[p] = tr.W[q];
            continue;
          }
          tr.distinct[p] = 1;
          const int slot = (int)cdf.size();
          tr.W[p] = slot_ptr(slot);
          cdf.push_back(reinterpret_cast<df32 *>(slot_ptr(slot)));
          img_m.push_back({m[0], m[1], m[2]});
          h_ia.push_back(m[0]);
          h_ib.push_back((int)(m[1] + No * m[2]));
          p_ia.push_back((int)(m[0] + No * m[1]));
          p_ib.push_back(m[2]);
        }
        trips.push_back(tr);
      }
  flush();
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
