// Bandwidth kernels: general index permutation with scale/accumulate, fill,
// axpby.  All are HBM-bound; accesses are coalesced on both sides (a 32x32
// shared-memory tile when the fastest index changes) and the per-element
// index arithmetic is reduced to one block-level decomposition.
#include <algorithm>

#include "internal.hpp"

namespace gbcc {
namespace {

constexpr int MAXD = 6;

struct PermDesc {
  int nrest;
  int64_t rlen[MAXD];
  int64_t rss[MAXD];  // src stride of rest dim
  int64_t rsd[MAXD];  // dst stride of rest dim
};

__device__ __forceinline__ void decompose(const PermDesc &d, int64_t r,
                                          int64_t &so, int64_t &dof) {
  so = 0;
  dof = 0;
  for (int k = 0; k < d.nrest; ++k) {
    const int64_t q = r / d.rlen[k];
    const int64_t c = r - q * d.rlen[k];
    so += c * d.rss[k];
    dof += c * d.rsd[k];
    r = q;
  }
}

__device__ __forceinline__ double combine(double alpha, double s, double beta,
                                          const double *dptr) {
  const double v = (alpha == 1.0) ? s : __dmul_rn(alpha, s);
  if (beta == 0.0) return v;
  const double o = (beta == 1.0) ? *dptr : __dmul_rn(beta, *dptr);
  return __dadd_rn(v, o);
}

// src dim 0 is also dst dim 0: contiguous runs of length L0 on both sides.
__global__ void perm_runs_kernel(const double *__restrict__ src,
                                 double *__restrict__ dst, int64_t L0,
                                 PermDesc d, double alpha, double beta) {
  __shared__ int64_t base[2];
  if (threadIdx.x == 0) decompose(d, blockIdx.x, base[0], base[1]);
  __syncthreads();
  const int64_t so = base[0], dof = base[1];
  for (int64_t x = (int64_t)blockIdx.y * blockDim.x + threadIdx.x; x < L0;
       x += (int64_t)gridDim.y * blockDim.x) {
    double *dp = dst + dof + x;
    *dp = combine(alpha, src[so + x], beta, dp);
  }
}

// src dim 0 (x) goes to dst stride sd0; src dim p (y, src stride ssp) becomes
// the dst fastest dim.
__global__ void perm_tile_kernel(const double *__restrict__ src,
                                 double *__restrict__ dst, int64_t L0,
                                 int64_t Lp, int64_t ssp, int64_t sd0,
                                 int64_t tiles_x, int64_t tiles_y, PermDesc d,
                                 double alpha, double beta) {
  __shared__ double tile[32][33];
  __shared__ int64_t base[2];
  int64_t b = blockIdx.x;
  const int64_t tx_ = b % tiles_x;
  b /= tiles_x;
  const int64_t ty_ = b % tiles_y;
  const int64_t r = b / tiles_y;
  if (threadIdx.x == 0 && threadIdx.y == 0) decompose(d, r, base[0], base[1]);
  __syncthreads();
  const int64_t so = base[0], dof = base[1];
  const int64_t x0 = tx_ * 32, y0 = ty_ * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int64_t y = y0 + ty + 8 * k, x = x0 + tx;
    if (x < L0 && y < Lp) tile[ty + 8 * k][tx] = src[so + x + y * ssp];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int64_t x = x0 + ty + 8 * k, y = y0 + tx;
    if (x < L0 && y < Lp) {
      double *dp = dst + dof + y + x * sd0;
      *dp = combine(alpha, tile[tx][ty + 8 * k], beta, dp);
    }
  }
}

__global__ void fill_kernel(double *p, int64_t n, double v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

__global__ void axpby_kernel(int64_t n, double a, const double *__restrict__ x,
                             double b, double *__restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = (a == 0.0) ? 0.0 : __dmul_rn(a, x[i]);
    if (b != 0.0) v = __dadd_rn(v, __dmul_rn(b, y[i]));
    y[i] = v;
  }
}

int grid_for(const Context &ctx, int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)std::max(ctx.sm_count, 1) * 16;
  return (int)std::max<int64_t>(1, std::min(g, cap));
}

}  // namespace

void fill(Context &ctx, double *p, int64_t n, double v) {
  if (n <= 0) return;
  fill_kernel<<<grid_for(ctx, n, 256), 256, 0, ctx.stream>>>(p, n, v);
  GBCC_CHECK_LAUNCH(ctx);
}

void copy(Context &ctx, double *dst, const double *src, int64_t n) {
  if (n <= 0 || dst == src) return;
  GBCC_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * n,
                            cudaMemcpyDeviceToDevice, ctx.stream));
}

void axpby(Context &ctx, int64_t n, double a, const double *x, double b,
           double *y) {
  if (n <= 0) return;
  axpby_kernel<<<grid_for(ctx, n, 256), 256, 0, ctx.stream>>>(n, a, x, b, y);
  GBCC_CHECK_LAUNCH(ctx);
}

void permute(Context &ctx, const Ten &src, const int *perm, double alpha,
             double beta, Ten &dst) {
  const int n = src.order;
  require(dst.order == n && n >= 1 && n <= MAXD, "permute: order mismatch");
  require(src.p != dst.p, "permute: in-place permutation is not supported");
  for (int q = 0; q < n; ++q)
    require(dst.lens[q] == src.lens[perm[q]], "permute: length mismatch");
  if (src.size() == 0) return;
  // strides
  int64_t ss[MAXD], ds[MAXD], sd[MAXD];
  int64_t acc = 1;
  for (int d = 0; d < n; ++d) { ss[d] = acc; acc *= src.lens[d]; }
  acc = 1;
  for (int q = 0; q < n; ++q) { ds[q] = acc; acc *= dst.lens[q]; }
  for (int q = 0; q < n; ++q) sd[perm[q]] = ds[q];
  // merge src dims d, d+1 that stay adjacent (and in order) in dst; drop len-1 dims
  struct Dim { int64_t len, ss, sd; };
  std::vector<Dim> dims;
  for (int d = 0; d < n; ++d) {
    if (src.lens[d] == 1) continue;
    Dim cur{src.lens[d], ss[d], sd[d]};
    if (!dims.empty()) {
      Dim &pv = dims.back();
      if (pv.ss * pv.len == cur.ss && pv.sd * pv.len == cur.sd) {
        pv.len *= cur.len;
        continue;
      }
    }
    dims.push_back(cur);
  }
  if (dims.empty()) dims.push_back(Dim{1, 1, 1});
  // identify the dst-fastest src dim
  int pfast = 0;
  for (size_t k = 0; k < dims.size(); ++k)
    if (dims[k].sd < dims[pfast].sd) pfast = (int)k;
  PermDesc d{};
  if (pfast == 0 && dims[0].ss == 1 && dims[0].sd == 1) {
    const int64_t L0 = dims[0].len;
    int64_t R = 1;
    d.nrest = 0;
    for (size_t k = 1; k < dims.size(); ++k) {
      d.rlen[d.nrest] = dims[k].len;
      d.rss[d.nrest] = dims[k].ss;
      d.rsd[d.nrest] = dims[k].sd;
      d.nrest++;
      R *= dims[k].len;
    }
    require(R < (1LL << 31), "permute: too many runs");
    const int threads = L0 >= 256 ? 256 : (L0 >= 128 ? 128 : (L0 >= 64 ? 64 : 32));
    int64_t gy = (L0 + threads - 1) / threads;
    if (gy > 65535) gy = 65535;
    dim3 grid((unsigned)R, (unsigned)gy);
    perm_runs_kernel<<<grid, threads, 0, ctx.stream>>>(src.p, dst.p, L0, d,
                                                       alpha, beta);
  } else {
    require(dims[0].ss == 1 && dims[pfast].sd == 1, "permute: stride logic");
    const int64_t L0 = dims[0].len, Lp = dims[pfast].len;
    int64_t R = 1;
    d.nrest = 0;
    for (size_t k = 1; k < dims.size(); ++k) {
      if ((int)k == pfast) continue;
      d.rlen[d.nrest] = dims[k].len;
      d.rss[d.nrest] = dims[k].ss;
      d.rsd[d.nrest] = dims[k].sd;
      d.nrest++;
      R *= dims[k].len;
    }
    const int64_t tx = (L0 + 31) / 32, ty = (Lp + 31) / 32;
    require(tx * ty * R < (1LL << 31), "permute: grid too large");
    perm_tile_kernel<<<(unsigned)(tx * ty * R), dim3(32, 8), 0, ctx.stream>>>(
        src.p, dst.p, L0, Lp, dims[pfast].ss, dims[0].sd, tx, ty, d, alpha,
        beta);
  }
  GBCC_CHECK_LAUNCH(ctx);
}

}  // namespace gbcc
