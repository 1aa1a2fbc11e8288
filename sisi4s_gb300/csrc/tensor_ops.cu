// Bandwidth kernels: general index permutation with scale/accumulate, fill,
// axpby.  All are HBM-bound; accesses are coalesced on both sides (a 32x32
// shared-memory tile when the fastest index changes) and the per-element
// index arithmetic is reduced to one block-level decomposition.
#include <algorithm>

#include "internal.hpp"

namespace gbcc {
namespace {

constexpr int MAXD = 6;

// dims of a permutation that are walked by block index (all but the one or
// two handled inside a block); lengths and run counts fit 32 bits (checked)
struct PermDesc {
  int nrest;
  unsigned rlen[MAXD];
  int64_t rss[MAXD];  // src stride of rest dim
  int64_t rsd[MAXD];  // dst stride of rest dim
};

// dst = alpha src + beta dst with alpha / beta classified on the host, so
// that only a real scaling or accumulation issues FP64 instructions
enum : int { ALPHA_ONE = 0, ALPHA_NEG = 1, ALPHA_GEN = 2 };
enum : int { BETA_ZERO = 0, BETA_ONE = 1, BETA_GEN = 2 };
struct Scale {
  int am, bm;
  double alpha, beta;
};

Scale make_scale(double alpha, double beta) {
  Scale s{};
  s.alpha = alpha;
  s.beta = beta;
  s.am = alpha == 1.0 ? ALPHA_ONE : (alpha == -1.0 ? ALPHA_NEG : ALPHA_GEN);
  s.bm = beta == 0.0 ? BETA_ZERO : (beta == 1.0 ? BETA_ONE : BETA_GEN);
  return s;
}

// same roundings as alpha * s (+ beta * d) with __dmul_rn / __dadd_rn;
// -s is the sign flip that __dmul_rn(-1, s) gives
__device__ __forceinline__ double apply(const Scale &sc, double s, const double *dptr) {
  double v;
  if (sc.am == ALPHA_ONE) v = s;
  else if (sc.am == ALPHA_NEG)
    v = __longlong_as_double(__double_as_longlong(s) ^ (long long)0x8000000000000000ull);
  else v = __dmul_rn(sc.alpha, s);
  if (sc.bm == BETA_ZERO) return v;
  const double o = (sc.bm == BETA_ONE) ? *dptr : __dmul_rn(sc.beta, *dptr);
  return __dadd_rn(v, o);
}

// 32-bit decomposition of a block's rest index (64-bit integer division
// costs FP64-pipe instructions on this GPU)
__device__ __forceinline__ void decompose(const PermDesc &d, unsigned r, int64_t &so,
                                          int64_t &dof) {
  so = 0;
  dof = 0;
  for (int k = 0; k < d.nrest; ++k) {
    const unsigned q = r / d.rlen[k];
    const unsigned c = r - q * d.rlen[k];
    so += (int64_t)c * d.rss[k];
    dof += (int64_t)c * d.rsd[k];
    r = q;
  }
}

// src dim 0 is also dst dim 0: contiguous runs of length L0 on both sides.
// A block moves an X x Y tile: X elements of the run (threadIdx.x) times Y
// consecutive indices of dim 1 (threadIdx.y; strides ss1 / sd1), with one
// decomposition of the remaining dims per block.
__global__ void perm_runs_kernel(const double *__restrict__ src, double *__restrict__ dst,
                                 int L0, int X, int nx, int L1, int Y, int ny,
                                 int64_t ss1, int64_t sd1, PermDesc d, Scale sc) {
  __shared__ int64_t base[2];
  unsigned b = blockIdx.x;
  const unsigned xt = b % nx;
  b /= nx;
  const unsigned yt = b % ny;
  const unsigned r = b / ny;
  if (threadIdx.x == 0 && threadIdx.y == 0) decompose(d, r, base[0], base[1]);
  __syncthreads();
  const int x0 = xt * X, x1 = min(L0, x0 + X);
  const int y0 = yt * Y, y1 = min(L1, y0 + Y);
  for (int y = y0 + threadIdx.y; y < y1; y += blockDim.y) {
    const double *sp = src + base[0] + (int64_t)y * ss1;
    double *dp = dst + base[1] + (int64_t)y * sd1;
    for (int x = x0 + threadIdx.x; x < x1; x += blockDim.x) dp[x] = apply(sc, sp[x], dp + x);
  }
}

// src dim 0 (x) goes to dst stride sd0; src dim p (y, src stride ssp) becomes
// the dst fastest dim: 32x32 shared tile, coalesced on both sides.
__global__ void perm_tile_kernel(const double *__restrict__ src,
                                 double *__restrict__ dst, int L0,
                                 int Lp, int64_t ssp, int64_t sd0,
                                 int tiles_x, int tiles_y, PermDesc d, Scale sc) {
  __shared__ double tile[32][33];
  __shared__ int64_t base[2];
  unsigned b = blockIdx.x;
  const unsigned tx_ = b % tiles_x;
  b /= tiles_x;
  const unsigned ty_ = b % tiles_y;
  const unsigned r = b / tiles_y;
  if (threadIdx.x == 0 && threadIdx.y == 0) decompose(d, r, base[0], base[1]);
  __syncthreads();
  const int64_t so = base[0], dof = base[1];
  const int x0 = tx_ * 32, y0 = ty_ * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int y = y0 + ty + 8 * k, x = x0 + tx;
    if (x < L0 && y < Lp) tile[ty + 8 * k][tx] = src[so + x + (int64_t)y * ssp];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int x = x0 + ty + 8 * k, y = y0 + tx;
    if (x < L0 && y < Lp) {
      double *dp = dst + dof + y + (int64_t)x * sd0;
      *dp = apply(sc, tile[tx][ty + 8 * k], dp);
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
  for (const Dim &dm : dims) require(dm.len < (1LL << 31), "permute: dimension too long");
  const Scale sc = make_scale(alpha, beta);
  PermDesc d{};
  auto add_rest = [&](const Dim &dm) {
    d.rlen[d.nrest] = (unsigned)dm.len;
    d.rss[d.nrest] = dm.ss;
    d.rsd[d.nrest] = dm.sd;
    d.nrest++;
    return dm.len;
  };
  if (pfast == 0 && dims[0].ss == 1 && dims[0].sd == 1) {
    const int L0 = (int)dims[0].len;
    const Dim d1 = dims.size() > 1 ? dims[1] : Dim{1, 0, 0};
    int64_t R = 1;
    for (size_t k = 2; k < dims.size(); ++k) R *= add_rest(dims[k]);
    // tile of X x Y elements per block, about 4096 elements
    const int X = std::min(L0, 4096);
    const int nx = (L0 + X - 1) / X;
    const int L1 = (int)d1.len;
    const int Y = (int)std::min<int64_t>(L1, std::max<int64_t>(1, 4096 / X));
    const int ny = (L1 + Y - 1) / Y;
    const int bx = X >= 256 ? 256 : (X >= 128 ? 128 : (X >= 64 ? 64 : 32));
    const int by = 256 / bx;
    require(R * nx * ny < (1LL << 31), "permute: too many blocks");
    perm_runs_kernel<<<(unsigned)(R * nx * ny), dim3(bx, by), 0, ctx.stream>>>(
        src.p, dst.p, L0, X, nx, L1, Y, ny, d1.ss, d1.sd, d, sc);
  } else {
    require(dims[0].ss == 1 && dims[pfast].sd == 1, "permute: stride logic");
    const int L0 = (int)dims[0].len, Lp = (int)dims[pfast].len;
    int64_t R = 1;
    for (size_t k = 1; k < dims.size(); ++k)
      if ((int)k != pfast) R *= add_rest(dims[k]);
    const int tx = (L0 + 31) / 32, ty = (Lp + 31) / 32;
    require((int64_t)tx * ty * R < (1LL << 31), "permute: grid too large");
    perm_tile_kernel<<<(unsigned)((int64_t)tx * ty * R), dim3(32, 8), 0, ctx.stream>>>(
        src.p, dst.p, L0, Lp, dims[pfast].ss, dims[0].sd, tx, ty, d, sc);
  }
  GBCC_CHECK_LAUNCH(ctx);
}

}  // namespace gbcc
