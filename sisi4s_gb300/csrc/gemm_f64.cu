// FP64 GEMM for sm_103a: C[M,N] = alpha op(A) op(B) + beta C, column-major.
//
// GB300 has no float64 kind for tcgen05.mma and a float64 rate far below its
// bf16 rate, so the plain-FP64 path is bound by the FP64 FMA pipe, not by
// HBM: a 64x64 block tile with 4x4 outputs per thread needs 0.25 bytes of
// shared memory per flop and ~0.03 bytes of global memory per flop, far below
// what the SM delivers.  The kernel therefore optimises for keeping the FP64
// pipe fed: operand tiles are staged in shared memory with a register
// prefetch of the next k-tile, so the global loads of tile k+1 overlap the
// FMAs of tile k.
#include "internal.hpp"

namespace gbcc {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

struct PtrBatch {
  const double *const *A;
  const double *const *B;
  double *const *C;
};

template <bool TA, bool TB>
__device__ __forceinline__ void load_tiles(const double *__restrict__ A,
                                           int64_t lda,
                                           const double *__restrict__ B,
                                           int64_t ldb, int64_t M, int64_t N,
                                           int64_t K, int64_t m0, int64_t n0,
                                           int64_t k0, double ra[4],
                                           double rb[4]) {
  const int t = threadIdx.x;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    int64_t m, k;
    if (!TA) {  // A(m,k) = A[m + k lda], m contiguous
      m = m0 + (t % 64);
      k = k0 + (t / 64) + 4 * r;
    } else {  // A(m,k) = A[k + m lda], k contiguous
      k = k0 + (t % 16);
      m = m0 + (t / 16) + 16 * r;
    }
    ra[r] = (m < M && k < K) ? (TA ? A[k + m * lda] : A[m + k * lda]) : 0.0;
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    int64_t n, k;
    if (!TB) {  // B(k,n) = B[k + n ldb], k contiguous
      k = k0 + (t % 16);
      n = n0 + (t / 16) + 16 * r;
    } else {  // B(k,n) = B[n + k ldb], n contiguous
      n = n0 + (t % 64);
      k = k0 + (t / 64) + 4 * r;
    }
    rb[r] = (n < N && k < K) ? (TB ? B[n + k * ldb] : B[k + n * ldb]) : 0.0;
  }
}

template <bool TA, bool TB>
__device__ __forceinline__ void store_tiles(double (*As)[BM + 1],
                                            double (*Bs)[BN + 1],
                                            const double ra[4],
                                            const double rb[4]) {
  const int t = threadIdx.x;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    int m, k;
    if (!TA) {
      m = t % 64;
      k = t / 64 + 4 * r;
    } else {
      k = t % 16;
      m = t / 16 + 16 * r;
    }
    As[k][m] = ra[r];
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    int n, k;
    if (!TB) {
      k = t % 16;
      n = t / 16 + 16 * r;
    } else {
      n = t % 64;
      k = t / 64 + 4 * r;
    }
    Bs[k][n] = rb[r];
  }
}

// Split-K: with fewer output tiles than the GPU has SMs, blockIdx.x also
// selects one of `ksplit` consecutive K ranges of `kchunk` (a multiple of
// BK); each writes its unscaled partial product to W[split][z][m + n M], and
// splitk_reduce_kernel sums the partials in split order (deterministic).
struct SplitK {
  int64_t ksplit = 1, kchunk = 0;
  double *W = nullptr;
};

template <bool TA, bool TB, bool PTR>
__global__ void __launch_bounds__(NT)
    dgemm_kernel(int64_t M, int64_t N, int64_t K, double alpha,
                 const double *__restrict__ A0, int64_t lda,
                 const double *__restrict__ B0, int64_t ldb, double beta,
                 double *__restrict__ C0, int64_t ldc, int64_t sA, int64_t sB,
                 int64_t sC, PtrBatch pb, int64_t tiles_m, SplitK sk) {
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  const int64_t z = blockIdx.z + (int64_t)gridDim.z * blockIdx.y;
  const double *A;
  const double *B;
  double *C;
  if (PTR) {
    A = pb.A[z];
    B = pb.B[z];
    C = pb.C[z];
  } else {
    A = A0 + z * sA;
    B = B0 + z * sB;
    C = C0 + z * sC;
  }
  const int64_t ntiles = (int64_t)gridDim.x / sk.ksplit;
  const int64_t split = blockIdx.x / ntiles;
  const int64_t tile = blockIdx.x - split * ntiles;
  const int64_t tm = tile % tiles_m;
  const int64_t tn = tile / tiles_m;
  const int64_t m0 = tm * BM, n0 = tn * BN;
  // this block's K range [kb, kend)
  const int64_t kb = sk.ksplit > 1 ? split * sk.kchunk : 0;
  const int64_t kend = sk.ksplit > 1 ? min(K, kb + sk.kchunk) : K;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  double ra[4], rb[4];
  load_tiles<TA, TB>(A, lda, B, ldb, M, N, kend, m0, n0, kb, ra, rb);
  for (int64_t k0 = kb; k0 < kend; k0 += BK) {
    store_tiles<TA, TB>(As, Bs, ra, rb);
    __syncthreads();
    if (k0 + BK < kend)
      load_tiles<TA, TB>(A, lda, B, ldb, M, N, kend, m0, n0, k0 + BK, ra, rb);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  if (sk.ksplit > 1) {
    double *w = sk.W + ((int64_t)split * gridDim.y * gridDim.z + z) * M * N;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t n = n0 + ty + 16 * j;
      if (n >= N) continue;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int64_t m = m0 + tx + 16 * i;
        if (m < M) w[m + n * M] = acc[i][j];
      }
    }
    return;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int64_t n = n0 + ty + 16 * j;
    if (n >= N) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t m = m0 + tx + 16 * i;
      if (m >= M) continue;
      double *c = C + m + n * ldc;
      double v = alpha * acc[i][j];
      if (beta != 0.0) v = fma(beta, *c, v);
      *c = v;
    }
  }
}

// C[z](m, n) = alpha sum_s W[s][z](m, n) + beta C[z](m, n), splits summed in
// order; one thread per output
template <bool PTR>
__global__ void splitk_reduce_kernel(int64_t M, int64_t N, int64_t nbatch, int64_t ks,
                                     const double *__restrict__ W, double alpha, double beta,
                                     double *__restrict__ C0, int64_t ldc, int64_t sC,
                                     PtrBatch pb) {
  const int64_t per = M * N;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < per * nbatch;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t z = e / per, r = e - z * per;
    const int64_t n = r / M, m = r - n * M;
    double s = 0.0;
    for (int64_t q = 0; q < ks; ++q) s += W[(q * nbatch + z) * per + r];
    double *c = (PTR ? pb.C[z] : C0 + z * sC) + m + n * ldc;
    double v = alpha * s;
    if (beta != 0.0) v = fma(beta, *c, v);
    *c = v;
  }
}

template <bool PTR>
void launch(Context &ctx, bool ta, bool tb, int64_t M, int64_t N, int64_t K,
            double alpha, const double *A, int64_t lda, const double *B,
            int64_t ldb, double beta, double *C, int64_t ldc, int64_t batch,
            int64_t sA, int64_t sB, int64_t sC, PtrBatch pb) {
  if (M <= 0 || N <= 0 || batch <= 0) return;
  const int64_t tiles_m = (M + BM - 1) / BM;
  const int64_t tiles_n = (N + BN - 1) / BN;
  require(tiles_m * tiles_n < (1LL << 31), "gemm: too many tiles");
  // batch split into grid.z (<= 65535) x grid.y
  int64_t gz = batch < 65535 ? batch : 65535;
  while (batch % gz) --gz;
  const int64_t gy = batch / gz;
  require(gy <= 65535, "gemm: batch too large");
  // split K when the tiles of all batch entries fill less than the GPU: aim
  // for ctx.f64_split_blocks blocks per SM (3 by default), every split at
  // least 4 k-tiles long
  SplitK sk;
  const int64_t G = std::max(ctx.sm_count, 1);
  const int64_t blocks = tiles_m * tiles_n * batch;
  DBuf wsp;
  if (ctx.f64_split_blocks > 0 && blocks < G && K >= 8 * BK) {
    int64_t ks = std::min<int64_t>((ctx.f64_split_blocks * G + blocks - 1) / blocks, 64);
    ks = std::min<int64_t>(ks, K / (4 * BK));
    if (ks > 1) {
      int64_t kchunk = (K + ks - 1) / ks;
      kchunk = (kchunk + BK - 1) / BK * BK;
      ks = (K + kchunk - 1) / kchunk;
      if (ks > 1) {
        sk.ksplit = ks;
        sk.kchunk = kchunk;
        wsp.alloc(ctx, sizeof(double) * ks * batch * M * N);
        sk.W = wsp.as<double>();
      }
    }
  }
  dim3 grid((unsigned)(tiles_m * tiles_n * sk.ksplit), (unsigned)gy, (unsigned)gz);
  auto k00 = dgemm_kernel<false, false, PTR>;
  auto k01 = dgemm_kernel<false, true, PTR>;
  auto k10 = dgemm_kernel<true, false, PTR>;
  auto k11 = dgemm_kernel<true, true, PTR>;
  auto kern = ta ? (tb ? k11 : k10) : (tb ? k01 : k00);
  kern<<<grid, NT, 0, ctx.stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C,
                                    ldc, sA, sB, sC, pb, tiles_m, sk);
  GBCC_CHECK_LAUNCH(ctx);
  if (sk.ksplit > 1) {
    const int64_t n = M * N * batch;
    const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, G * 8));
    splitk_reduce_kernel<PTR><<<g, 256, 0, ctx.stream>>>(M, N, batch, sk.ksplit, sk.W, alpha,
                                                          beta, C, ldc, sC, pb);
    GBCC_CHECK_LAUNCH(ctx);
  }
  ctx.flops += 2.0 * (double)M * (double)N * (double)K * (double)batch;
}

// ------------------------------------------------------------------ GEMV
// y[i] = alpha * sum_k A(i, k) x[k] + beta * y[i], FP64, deterministic.
// A(i, k) = A[i * ars + k * aks], x[k] = x[k * incx], y[i] = y[i * incy].
// The GEMV shapes of the CCSD iteration (one index of length 1) are bound by
// the FP64 FMA pipe and HBM, not by tensor cores, so they stay in FP64.
//
// Rows contiguous in k (aks == 1): one warp per output, lanes stride over k,
// shuffle reduction in a fixed order.
__global__ void gemv_rows_kernel(int64_t Mo, int64_t K, double alpha,
                                 const double *__restrict__ A, int64_t ars,
                                 const double *__restrict__ x, int64_t incx,
                                 double beta, double *__restrict__ y, int64_t incy) {
  const int lane = threadIdx.x % 32;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; i < Mo;
       i += (int64_t)gridDim.x * blockDim.x / 32) {
    const double *a = A + i * ars;
    double s = 0.0;
    for (int64_t k = lane; k < K; k += 32) s = fma(a[k], x[k * incx], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) {
      double v = alpha * s;
      if (beta != 0.0) v = fma(beta, y[i * incy], v);
      y[i * incy] = v;
    }
  }
}

// Outputs contiguous (ars == 1): threads over i (coalesced), blockIdx.y over
// K-chunks; partials [kchunks][Mo] are summed in chunk order afterwards.
__global__ void gemv_cols_kernel(int64_t Mo, int64_t K, int64_t kchunk,
                                 const double *__restrict__ A, int64_t aks,
                                 const double *__restrict__ x, int64_t incx,
                                 double *__restrict__ part) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Mo) return;
  const int64_t k0 = (int64_t)blockIdx.y * kchunk, k1 = min(K, k0 + kchunk);
  double s = 0.0;
  for (int64_t k = k0; k < k1; ++k) s = fma(A[i + k * aks], x[k * incx], s);
  part[(int64_t)blockIdx.y * Mo + i] = s;
}

__global__ void gemv_sum_kernel(int64_t Mo, int nparts, const double *__restrict__ part,
                                double alpha, double beta, double *__restrict__ y,
                                int64_t incy) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Mo;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < nparts; ++c) s += part[(int64_t)c * Mo + i];
    double v = alpha * s;
    if (beta != 0.0) v = fma(beta, y[i * incy], v);
    y[i * incy] = v;
  }
}

void gemv(Context &ctx, int64_t Mo, int64_t K, double alpha, const double *A,
          int64_t ars, int64_t aks, const double *x, int64_t incx, double beta,
          double *y, int64_t incy) {
  const int64_t G = std::max(ctx.sm_count, 1);
  // a single output (a dot product) goes to the K-split form below, whatever
  // the layout: one warp over all of K would leave the GPU idle
  if (aks == 1 && Mo > 1) {
    const int64_t blocks = std::min<int64_t>((Mo * 32 + 255) / 256, G * 32);
    gemv_rows_kernel<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, ctx.stream>>>(
        Mo, K, alpha, A, ars, x, incx, beta, y, incy);
    GBCC_CHECK_LAUNCH(ctx);
    return;
  }
  // with one output the row stride is never used (row 0 only)
  require(ars == 1 || Mo == 1, "gemv: one operand index must be contiguous");
  const int64_t bx = (Mo + 255) / 256;
  int64_t nch = std::max<int64_t>(1, std::min<int64_t>((G * 8 + bx - 1) / bx, (K + 63) / 64));
  nch = std::min<int64_t>(nch, 65535);
  const int64_t kchunk = (K + nch - 1) / nch;
  nch = (K + kchunk - 1) / kchunk;
  DBuf part(ctx, sizeof(double) * Mo * nch);
  gemv_cols_kernel<<<dim3((unsigned)bx, (unsigned)nch), 256, 0, ctx.stream>>>(
      Mo, K, kchunk, A, aks, x, incx, part.as<double>());
  GBCC_CHECK_LAUNCH(ctx);
  gemv_sum_kernel<<<(unsigned)std::min<int64_t>(bx, G * 8), 256, 0, ctx.stream>>>(
      Mo, (int)nch, part.as<double>(), alpha, beta, y, incy);
  GBCC_CHECK_LAUNCH(ctx);
}

}  // namespace

void gemm_f64(Context &ctx, bool ta, bool tb, int64_t M, int64_t N, int64_t K,
              double alpha, const double *A, int64_t lda, const double *B,
              int64_t ldb, double beta, double *C, int64_t ldc, int64_t batch,
              int64_t sA, int64_t sB, int64_t sC) {
  if (K == 0) {
    // C = beta C
    require(batch == 1 || sC >= ldc * N, "gemm: K=0 with overlapping batch");
    for (int64_t z = 0; z < batch; ++z)
      for (int64_t n = 0; n < N; ++n)
        axpby(ctx, M, 0.0, C + z * sC + n * ldc, beta, C + z * sC + n * ldc);
    return;
  }
  launch<false>(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc,
                batch, sA, sB, sC, PtrBatch{nullptr, nullptr, nullptr});
}

void gemm_f64_ptr(Context &ctx, bool ta, bool tb, int64_t M, int64_t N,
                  int64_t K, double alpha, const double *const *A, int64_t lda,
                  const double *const *B, int64_t ldb, double beta,
                  double *const *C, int64_t ldc, int64_t batch) {
  require(K > 0, "gemm_f64_ptr: K must be positive");
  launch<true>(ctx, ta, tb, M, N, K, alpha, nullptr, lda, nullptr, ldb, beta,
               nullptr, ldc, batch, 0, 0, 0, PtrBatch{A, B, C});
}

void gemm(Context &ctx, bool ta, bool tb, int64_t M, int64_t N, int64_t K,
          double alpha, const double *A, int64_t lda, const double *B,
          int64_t ldb, double beta, double *C, int64_t ldc, int64_t batch,
          int64_t sA, int64_t sB, int64_t sC, int precision) {
  const double fl = 2.0 * (double)M * (double)N * (double)K * (double)batch;
  if (batch == 1 && K > 0 && (M == 1 || N == 1)) {
    // matrix-vector product: FP64 GEMV (both precision modes)
    if (N == 1) {  // C[i,0] = sum_k op(A)(i,k) op(B)(k,0)
      gemv(ctx, M, K, alpha, A, ta ? lda : 1, ta ? 1 : lda, B, tb ? ldb : 1, beta, C, 1);
    } else {       // C[0,j] = sum_k op(B)(k,j) op(A)(0,k)
      gemv(ctx, N, K, alpha, B, tb ? 1 : ldb, tb ? ldb : 1, A, ta ? 1 : lda, beta, C, ldc);
    }
    ctx.flops += fl;
    return;
  }
  // the tensor-core threshold is per batch entry, so that a product takes the
  // same precision route alone and inside a batch of systems
  if (precision == GBCC_PREC_EMU && K > 0 && fl / (double)batch >= ctx.emu_min_flops) {
    gemm_emu(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, batch,
             sA, sB, sC);
    return;
  }
  gemm_f64(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, batch,
           sA, sB, sC);
}

}  // namespace gbcc
