// Bandwidth kernels of the CCSD iteration (all FP64, all deterministic).
//
// Amplitudes, residua and DIIS history are stored as one "Fock vector"
// buffer per object: T1[Nv,No] at offset 0, zero padding, T2[Nv,Nv,No,No] at
// offset off2 (a multiple of 32 doubles).  Elementwise arithmetic uses
// explicit _rn intrinsics (no FMA contraction) in the order of the reference
// statements, so these kernels reproduce the CPU restatement bit for bit.
// Reductions write one partial per block into a fixed-size array that a
// single block then sums in a fixed order: the result depends only on the
// problem size, never on timing or on other work sharing the GPU.
#include "ccsd_kernels.hpp"

namespace gbcc {
namespace {

constexpr int RT = 256;  // reduction block size

__device__ __forceinline__ double block_sum(double v, double *sm) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  __syncthreads();
  if (l == 0) sm[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = (threadIdx.x < blockDim.x / 32) ? sm[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

__global__ void outer_add_kernel(double *__restrict__ X,
                                 const double *__restrict__ T2,
                                 const double *__restrict__ T1, double c,
                                 int64_t Nv, int64_t No, int64_t nz) {
  // nz systems of one shape, each contiguous (X, T2: n apart; T1: Nv No)
  const int64_t n = Nv * Nv * No * No;
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < n * nz;
       f += (int64_t)gridDim.x * blockDim.x) {
    const int64_t z = f / n;
    const int64_t e = f - z * n;
    const double *t1 = T1 + z * Nv * No;
    int64_t r = e;
    const int64_t a = r % Nv; r /= Nv;
    const int64_t b = r % Nv; r /= Nv;
    const int64_t i = r % No;
    const int64_t j = r / No;
    double p = __dmul_rn(t1[a + Nv * i], t1[b + Nv * j]);
    if (c != 1.0) p = __dmul_rn(c, p);
    X[f] = __dadd_rn(T2[f], p);
  }
}

// Jacobi update of one Fock vector + fused reductions.
// est = -(R - s T)/(D + s), dT = est - T.  Partial sums per block:
//   [0] dT.dT, [1] est.est, [2 + q] dT.hist[q] for q < nhist.
struct UpdArgs {
  const double *R, *T;
  double *est, *dT;
  const double *eps_h, *eps_p;
  double shift;
  int64_t Nv, No, n1, off2, ntot;
  int nhist;
  const double *hist[GBCC_MAX_DIIS];
  double *partials;  // [gridDim.x][2 + nhist]
};

__global__ void update_kernel(UpdArgs a) {
  __shared__ double sm[32];
  double acc[2 + GBCC_MAX_DIIS];
#pragma unroll
  for (int q = 0; q < 2 + GBCC_MAX_DIIS; ++q) acc[q] = 0.0;
  const int64_t n2 = a.Nv * a.Nv * a.No * a.No;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < a.ntot;
       e += (int64_t)gridDim.x * blockDim.x) {
    double d;
    if (e < a.n1) {
      const int64_t av = e % a.Nv, iv = e / a.Nv;
      d = __dsub_rn(a.eps_p[av], a.eps_h[iv]);
    } else if (e >= a.off2 && e < a.off2 + n2) {
      int64_t r = e - a.off2;
      const int64_t av = r % a.Nv; r /= a.Nv;
      const int64_t bv = r % a.Nv; r /= a.Nv;
      const int64_t iv = r % a.No;
      const int64_t jv = r / a.No;
      d = __dsub_rn(__dadd_rn(__dsub_rn(a.eps_p[av], a.eps_h[iv]), a.eps_p[bv]),
                    a.eps_h[jv]);
    } else {
      a.est[e] = 0.0;
      a.dT[e] = 0.0;
      continue;
    }
    const double t = a.T[e];
    double r = a.R[e];
    if (a.shift != 0.0) r = __dsub_rn(r, __dmul_rn(a.shift, t));
    const double est = __ddiv_rn(-r, __dadd_rn(d, a.shift));
    const double dt = __dsub_rn(est, t);
    a.est[e] = est;
    a.dT[e] = dt;
    acc[0] = fma(dt, dt, acc[0]);
    acc[1] = fma(est, est, acc[1]);
    for (int q = 0; q < a.nhist; ++q) acc[2 + q] = fma(dt, a.hist[q][e], acc[2 + q]);
  }
  const int nq = 2 + a.nhist;
  for (int q = 0; q < nq; ++q) {
    const double s = block_sum(acc[q], sm);
    if (threadIdx.x == 0) a.partials[(int64_t)blockIdx.x * nq + q] = s;
  }
}

// sums partials[nblk][nq] -> out[q] in a fixed order (one block)
__global__ void finalize_kernel(const double *__restrict__ partials, int nblk,
                                int nq, double *__restrict__ out) {
  __shared__ double sm[32];
  for (int q = 0; q < nq; ++q) {
    double v = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += partials[(int64_t)b * nq + q];
    const double s = block_sum(v, sm);
    if (threadIdx.x == 0) out[q] = s;
  }
}

// energy partials: [0] T2.V  [1] T1T1.V  [2] T2.Vx  [3] T1T1.Vx
__global__ void energy_kernel(const double *__restrict__ T1,
                              const double *__restrict__ T2,
                              const double *__restrict__ V,
                              const double *__restrict__ Vx, int64_t Nv,
                              int64_t No, double *__restrict__ partials) {
  __shared__ double sm[32];
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const int64_t n = Nv * Nv * No * No;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = e;
    const int64_t a = r % Nv; r /= Nv;
    const int64_t b = r % Nv; r /= Nv;
    const int64_t i = r % No;
    const int64_t j = r / No;
    const double tt = __dmul_rn(T1[a + Nv * i], T1[b + Nv * j]);
    const double t2 = T2[e], v = V[e], vx = Vx[e];
    acc[0] = fma(t2, v, acc[0]);
    acc[1] = fma(tt, v, acc[1]);
    acc[2] = fma(t2, vx, acc[2]);
    acc[3] = fma(tt, vx, acc[3]);
  }
  for (int q = 0; q < 4; ++q) {
    const double s = block_sum(acc[q], sm);
    if (threadIdx.x == 0) partials[(int64_t)blockIdx.x * 4 + q] = s;
  }
}

// PairEnergy[i,j] (ClusterSinglesDoublesAlgorithm.cxx:227-232), one block per (i,j)
__global__ void pair_energy_kernel(const double *__restrict__ T1,
                                   const double *__restrict__ T2,
                                   const double *__restrict__ V,
                                   const double *__restrict__ Vx, int64_t Nv,
                                   int64_t No, double *__restrict__ out) {
  __shared__ double sm[32];
  const int64_t i = blockIdx.x % No, j = blockIdx.x / No;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const int64_t base = Nv * Nv * (i + No * j);
  for (int64_t ab = threadIdx.x; ab < Nv * Nv; ab += blockDim.x) {
    const int64_t a = ab % Nv, b = ab / Nv;
    const double tt = __dmul_rn(T1[a + Nv * i], T1[b + Nv * j]);
    const double t2 = T2[base + ab], v = V[base + ab], vx = Vx[base + ab];
    acc[0] = fma(t2, v, acc[0]);
    acc[1] = fma(t2, vx, acc[1]);
    acc[2] = fma(tt, v, acc[2]);
    acc[3] = fma(tt, vx, acc[3]);
  }
  double s[4];
  for (int q = 0; q < 4; ++q) s[q] = block_sum(acc[q], sm);
  if (threadIdx.x == 0)
    out[i + No * j] = 2.0 * s[0] + (-1.0) * s[1] + 2.0 * s[2] + (-1.0) * s[3];
}

// DIIS: write 2<dT_i, dT> into row/column k+1 of B, solve the leading
// (count+1) block B c = (-1,0,...,0) by Gaussian elimination with partial
// pivoting, and emit the weights w_j = c[i_j + 1], i_j = (k + N - j) % N.
struct HistSlots {
  int n;
  int slot[GBCC_MAX_DIIS];
};

__global__ void diis_solve_kernel(double *B, int N, int k, int count,
                                  const double *__restrict__ sums,
                                  HistSlots hs, double *weights,
                                  double *lambda, int *status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int ld = N + 1;
  // sums: [0] dT.dT (own slot), [2+q] dT.hist[q] (slot hs.slot[q])
  B[(k + 1) + ld * (k + 1)] = 2.0 * sums[0];
  for (int q = 0; q < hs.n; ++q) {
    const int i = hs.slot[q];
    const double ov = 2.0 * sums[2 + q];
    B[(k + 1) + ld * (i + 1)] = ov;
    B[(i + 1) + ld * (k + 1)] = ov;
  }
  const int dim = count + 1;
  double M[(GBCC_MAX_DIIS + 1) * (GBCC_MAX_DIIS + 1)];
  double x[GBCC_MAX_DIIS + 1];
  for (int c = 0; c < dim; ++c)
    for (int r = 0; r < dim; ++r) M[r + dim * c] = B[r + ld * c];
  for (int r = 0; r < dim; ++r) x[r] = (r == 0) ? -1.0 : 0.0;
  int st = 0;
  for (int c = 0; c < dim; ++c) {
    int piv = c;
    double best = fabs(M[c + dim * c]);
    for (int r = c + 1; r < dim; ++r)
      if (fabs(M[r + dim * c]) > best) { best = fabs(M[r + dim * c]); piv = r; }
    if (!isfinite(best)) { st = 2; break; }  // overflowed overlaps
    if (!(best > 0.0)) { st = 1; break; }     // exact zero pivot
    if (piv != c) {
      for (int cc = 0; cc < dim; ++cc) {
        const double t = M[c + dim * cc];
        M[c + dim * cc] = M[piv + dim * cc];
        M[piv + dim * cc] = t;
      }
      const double t = x[c]; x[c] = x[piv]; x[piv] = t;
    }
    const double inv = 1.0 / M[c + dim * c];
    for (int r = c + 1; r < dim; ++r) {
      const double f = M[r + dim * c] * inv;
      if (f == 0.0) continue;
      for (int cc = c; cc < dim; ++cc) M[r + dim * cc] -= f * M[c + dim * cc];
      x[r] -= f * x[c];
    }
  }
  if (!st) {
    for (int r = dim - 1; r >= 0; --r) {
      double s = x[r];
      for (int cc = r + 1; cc < dim; ++cc) s -= M[r + dim * cc] * x[cc];
      x[r] = s / M[r + dim * r];
      if (!isfinite(x[r])) st = 2;
    }
  }
  *status = st;
  *lambda = st ? 0.0 : x[0];
  for (int j = 0; j < count; ++j) {
    const int i = (k + N - j) % N;
    weights[j] = st ? (j == 0 ? 1.0 : 0.0) : x[i + 1];
  }
}

// next = sum_j w_j A_j (j = 0..count-1, added one scaled term at a time from
// zero, DiisMixer.cxx:160-174) + partial sums of next.next
struct CombArgs {
  int count;
  const double *src[GBCC_MAX_DIIS];
  const double *w;
  double *out;
  int64_t n;
  double *partials;
};

__global__ void combine_kernel(CombArgs a) {
  __shared__ double sm[32];
  double acc = 0.0;
  double w[GBCC_MAX_DIIS];
  for (int j = 0; j < a.count; ++j) w[j] = a.w[j];
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < a.n;
       e += (int64_t)gridDim.x * blockDim.x) {
    double v = 0.0;
    for (int j = 0; j < a.count; ++j) v = __dadd_rn(v, __dmul_rn(w[j], a.src[j][e]));
    a.out[e] = v;
    acc = fma(v, v, acc);
  }
  const double s = block_sum(acc, sm);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = s;
}

// LinearMixer::append (LinearMixer.cxx:30-44) on (next, nres) with the last
// pair: last *= 1-r; next *= r; next += last (same for the residua), plus
// partial sums [0] nres.nres [1] next.next
__global__ void linear_mix_kernel(double *__restrict__ next,
                                  double *__restrict__ nres,
                                  double *__restrict__ last,
                                  double *__restrict__ lres, double r,
                                  int64_t n, double *__restrict__ partials) {
  __shared__ double sm[32];
  double a0 = 0.0, a1 = 0.0;
  const double q = 1.0 - r;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double l = __dmul_rn(last[e], q);
    const double nx = __dadd_rn(__dmul_rn(next[e], r), l);
    const double lr = __dmul_rn(lres[e], q);
    const double nr = __dadd_rn(__dmul_rn(nres[e], r), lr);
    last[e] = l;
    lres[e] = lr;
    next[e] = nx;
    nres[e] = nr;
    a0 = fma(nr, nr, a0);
    a1 = fma(nx, nx, a1);
  }
  const double s0 = block_sum(a0, sm);
  const double s1 = block_sum(a1, sm);
  if (threadIdx.x == 0) {
    partials[blockIdx.x * 2 + 0] = s0;
    partials[blockIdx.x * 2 + 1] = s1;
  }
}

// sliceIntoResiduum (ClusterSinglesDoublesAlgorithm.cxx:888-915):
// R[a0+x, b0+y, i, j] += Rxy[x,y,i,j]; if mirror: R[b0+y, a0+x, j, i] += Rxy[x,y,i,j]
__global__ void slice_add_kernel(double *__restrict__ R,
                                 const double *__restrict__ Rxy, int64_t Nv,
                                 int64_t No, int64_t a0, int64_t b0,
                                 int64_t nx, int64_t ny, int mirror, int64_t nz) {
  const int64_t n = nx * ny * No * No;
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < n * nz;
       f += (int64_t)gridDim.x * blockDim.x) {
    const int64_t z = f / n;
    const int64_t e = f - z * n;
    double *Rz = R + z * Nv * Nv * No * No;
    int64_t r = e;
    const int64_t x = r % nx; r /= nx;
    const int64_t y = r % ny; r /= ny;
    const int64_t i = r % No;
    const int64_t j = r / No;
    const double v = Rxy[f];
    double *p = Rz + (a0 + x) + Nv * ((b0 + y) + Nv * (i + No * j));
    *p = __dadd_rn(*p, v);
    if (mirror) {
      double *q = Rz + (b0 + y) + Nv * ((a0 + x) + Nv * (j + No * i));
      *q = __dadd_rn(*q, v);
    }
  }
}

// gather slice [G, x0:x0+nx, :] of a [G, Nv, Nv] tensor into [G, nx, Nv],
// for nz systems of one shape stored one after another
__global__ void gather_slice_kernel(double *__restrict__ dst,
                                    const double *__restrict__ src, int64_t G,
                                    int64_t Nv, int64_t x0, int64_t nx, int64_t nz) {
  const int64_t n = G * nx * Nv;
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < n * nz;
       f += (int64_t)gridDim.x * blockDim.x) {
    const int64_t z = f / n;
    int64_t r = f - z * n;
    const int64_t g = r % G; r /= G;
    const int64_t x = r % nx;
    const int64_t c = r / nx;
    dst[f] = src[z * G * Nv * Nv + g + G * ((x0 + x) + Nv * c)];
  }
}

// systems of one shape side by side: gather dst[z n + e] = src[z][e],
// scatter dst[z][e] = src[z n + e] (the per-system pointers in device memory)
__global__ void batch_gather_kernel(const double *const *__restrict__ src, int64_t n,
                                    int64_t nz, double *__restrict__ dst) {
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < n * nz;
       f += (int64_t)gridDim.x * blockDim.x) {
    const int64_t z = f / n;
    dst[f] = src[z][f - z * n];
  }
}

__global__ void batch_scatter_kernel(const double *__restrict__ src, int64_t n, int64_t nz,
                                     double *const *__restrict__ dst) {
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < n * nz;
       f += (int64_t)gridDim.x * blockDim.x) {
    const int64_t z = f / n;
    dst[z][f - z * n] = src[f];
  }
}

// contiguous copy of the sub-block [G, p0:p0+np, q0:q0+nq] of Gamma[G,Np,Np]
__global__ void vertex_block_kernel(double *__restrict__ dst,
                                    const double *__restrict__ src, int64_t G,
                                    int64_t Np, int64_t p0, int64_t np,
                                    int64_t q0, int64_t nq) {
  const int64_t n = G * np * nq;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = e;
    const int64_t g = r % G; r /= G;
    const int64_t p = r % np;
    const int64_t q = r / np;
    dst[e] = src[g + G * ((p0 + p) + Np * (q0 + q))];
  }
}

__global__ void nonzero_kernel(const double *__restrict__ p, int64_t n,
                               int *__restrict__ flag) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    if (p[e] != 0.0) { *flag = 1; return; }
}

int ew_grid(const Context &ctx, int64_t n) {
  int64_t g = (n + 255) / 256;
  const int64_t cap = (int64_t)(ctx.sm_count > 0 ? ctx.sm_count : 148) * 8;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace

int reduction_blocks(const Context &ctx, int64_t n) {
  // depends on n only (and the device's SM count), never on timing
  int64_t g = (n + RT * 4 - 1) / (RT * 4);
  const int64_t cap = (int64_t)(ctx.sm_count > 0 ? ctx.sm_count : 148) * 4;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

void outer_add(Context &ctx, double *X, const double *T2, const double *T1,
               double c, int64_t Nv, int64_t No, int64_t nz) {
  outer_add_kernel<<<ew_grid(ctx, Nv * Nv * No * No * nz), 256, 0, ctx.stream>>>(
      X, T2, T1, c, Nv, No, nz);
  GBCC_CHECK_LAUNCH(ctx);
}

void jacobi_update(Context &ctx, const FockLayout &L, const double *R,
                   const double *T, double *est, double *dT,
                   const double *eps_h, const double *eps_p, double shift,
                   int nhist, const double *const *hist, double *partials,
                   double *sums) {
  UpdArgs a{};
  a.R = R; a.T = T; a.est = est; a.dT = dT;
  a.eps_h = eps_h; a.eps_p = eps_p; a.shift = shift;
  a.Nv = L.Nv; a.No = L.No; a.n1 = L.n1; a.off2 = L.off2; a.ntot = L.ntot;
  require(nhist <= GBCC_MAX_DIIS, "too many DIIS vectors");
  a.nhist = nhist;
  for (int q = 0; q < nhist; ++q) a.hist[q] = hist[q];
  a.partials = partials;
  const int nb = reduction_blocks(ctx, L.ntot);
  update_kernel<<<nb, RT, 0, ctx.stream>>>(a);
  GBCC_CHECK_LAUNCH(ctx);
  finalize_kernel<<<1, RT, 0, ctx.stream>>>(partials, nb, 2 + nhist, sums);
  GBCC_CHECK_LAUNCH(ctx);
}

void energy_terms(Context &ctx, const double *T1, const double *T2,
                  const double *V, const double *Vx, int64_t Nv, int64_t No,
                  double *partials, double *sums4) {
  const int nb = reduction_blocks(ctx, Nv * Nv * No * No);
  energy_kernel<<<nb, RT, 0, ctx.stream>>>(T1, T2, V, Vx, Nv, No, partials);
  GBCC_CHECK_LAUNCH(ctx);
  finalize_kernel<<<1, RT, 0, ctx.stream>>>(partials, nb, 4, sums4);
  GBCC_CHECK_LAUNCH(ctx);
}

void pair_energy(Context &ctx, const double *T1, const double *T2,
                 const double *V, const double *Vx, int64_t Nv, int64_t No,
                 double *out) {
  pair_energy_kernel<<<(unsigned)(No * No), RT, 0, ctx.stream>>>(T1, T2, V, Vx,
                                                                 Nv, No, out);
  GBCC_CHECK_LAUNCH(ctx);
}

void diis_solve(Context &ctx, double *B, int N, int k, int count,
                const double *sums, int nhist, const int *hist_slot,
                double *weights, double *lambda, int *status) {
  require(nhist <= GBCC_MAX_DIIS, "too many DIIS vectors");
  HistSlots hs{};
  hs.n = nhist;
  for (int q = 0; q < nhist; ++q) hs.slot[q] = hist_slot[q];
  diis_solve_kernel<<<1, 32, 0, ctx.stream>>>(B, N, k, count, sums, hs, weights,
                                              lambda, status);
  GBCC_CHECK_LAUNCH(ctx);
}

void diis_combine(Context &ctx, int count, const double *const *src,
                  const double *w, double *out, int64_t n, double *partials,
                  double *sum) {
  CombArgs a{};
  a.count = count;
  for (int j = 0; j < count; ++j) a.src[j] = src[j];
  a.w = w; a.out = out; a.n = n; a.partials = partials;
  const int nb = reduction_blocks(ctx, n);
  combine_kernel<<<nb, RT, 0, ctx.stream>>>(a);
  GBCC_CHECK_LAUNCH(ctx);
  finalize_kernel<<<1, RT, 0, ctx.stream>>>(partials, nb, 1, sum);
  GBCC_CHECK_LAUNCH(ctx);
}

void linear_mix(Context &ctx, double *next, double *nres, double *last,
                double *lres, double ratio, int64_t n, double *partials,
                double *sums2) {
  const int nb = reduction_blocks(ctx, n);
  linear_mix_kernel<<<nb, RT, 0, ctx.stream>>>(next, nres, last, lres, ratio,
                                               n, partials);
  GBCC_CHECK_LAUNCH(ctx);
  finalize_kernel<<<1, RT, 0, ctx.stream>>>(partials, nb, 2, sums2);
  GBCC_CHECK_LAUNCH(ctx);
}

void slice_add(Context &ctx, double *R, const double *Rxy, int64_t Nv,
               int64_t No, int64_t a0, int64_t b0, int64_t nx, int64_t ny,
               bool mirror, int64_t nz) {
  slice_add_kernel<<<ew_grid(ctx, nx * ny * No * No * nz), 256, 0, ctx.stream>>>(
      R, Rxy, Nv, No, a0, b0, nx, ny, mirror ? 1 : 0, nz);
  GBCC_CHECK_LAUNCH(ctx);
}

void gather_slice(Context &ctx, double *dst, const double *src, int64_t G,
                  int64_t Nv, int64_t x0, int64_t nx, int64_t nz) {
  gather_slice_kernel<<<ew_grid(ctx, G * nx * Nv * nz), 256, 0, ctx.stream>>>(
      dst, src, G, Nv, x0, nx, nz);
  GBCC_CHECK_LAUNCH(ctx);
}

void batch_gather(Context &ctx, const double *const *src_dev, int64_t n, int64_t nz,
                  double *dst) {
  batch_gather_kernel<<<ew_grid(ctx, n * nz), 256, 0, ctx.stream>>>(src_dev, n, nz, dst);
  GBCC_CHECK_LAUNCH(ctx);
}

void batch_scatter(Context &ctx, const double *src, int64_t n, int64_t nz,
                   double *const *dst_dev) {
  batch_scatter_kernel<<<ew_grid(ctx, n * nz), 256, 0, ctx.stream>>>(src, n, nz, dst_dev);
  GBCC_CHECK_LAUNCH(ctx);
}

void vertex_block(Context &ctx, double *dst, const double *src, int64_t G,
                  int64_t Np, int64_t p0, int64_t np, int64_t q0, int64_t nq) {
  vertex_block_kernel<<<ew_grid(ctx, G * np * nq), 256, 0, ctx.stream>>>(
      dst, src, G, Np, p0, np, q0, nq);
  GBCC_CHECK_LAUNCH(ctx);
}

void any_nonzero(Context &ctx, const double *p, int64_t n, int *flag_dev) {
  GBCC_CUDA(cudaMemsetAsync(flag_dev, 0, sizeof(int), ctx.stream));
  nonzero_kernel<<<ew_grid(ctx, n), 256, 0, ctx.stream>>>(p, n, flag_dev);
  GBCC_CHECK_LAUNCH(ctx);
}

}  // namespace gbcc
