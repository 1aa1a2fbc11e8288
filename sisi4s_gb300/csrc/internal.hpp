// Internal declarations of libgbcc: context, device tensors, launch helpers
// and the contraction engine.  Not part of the ABI.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <map>
#include <memory>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gbcc.h"

namespace gbcc {

// Thrown inside the library and turned into a gbcc_status at the ABI.
struct Error : std::runtime_error {
  gbcc_status status;
  Error(gbcc_status s, const std::string &m) : std::runtime_error(m), status(s) {}
};

#define GBCC_CUDA(call)                                                        \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      throw ::gbcc::Error(e_ == cudaErrorMemoryAllocation ? GBCC_OOM           \
                                                          : GBCC_CUDA_ERROR,   \
                          std::string(#call) + ": " + cudaGetErrorString(e_)); \
    }                                                                          \
  } while (0)

#define GBCC_CHECK_LAUNCH(ctx)                                                 \
  do {                                                                         \
    (ctx).launches++;                                                          \
    cudaError_t e_ = cudaGetLastError();                                       \
    if (e_ != cudaSuccess)                                                     \
      throw ::gbcc::Error(GBCC_CUDA_ERROR,                                     \
                          std::string("launch: ") + cudaGetErrorString(e_));   \
  } while (0)

inline void require(bool ok, const std::string &msg) {
  if (!ok) throw Error(GBCC_BAD_ARG, msg);
}

struct EmuPanels;

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string last_error;
  uint64_t launches = 0;
  double flops = 0.0;     // FP64-equivalent flops issued to GEMMs
  int sm_count = 0;
  // emulated-GEMM configuration
  int emu_slices = 6;
  // GEMMs smaller than this many flops stay in FP64 in precision mode
  double emu_min_flops = 1e7;
  // K-split policies: an FP64 GEMM whose output tiles fill less than the GPU
  // splits K to reach about this many blocks per SM (0: never splits); an
  // emulated GEMM splits K into at most this many parts (1: never)
  int f64_split_blocks = 3;
  int emu_max_ksplit = 64;
  // replay steady-state CCSD iterations as captured CUDA graphs
  bool use_graphs = true;
  // (T): distinct triple images whose W products share one batch (one W
  // slot of Nv^3 doubles each); 0 = from the free device memory
  int triples_batch_images = 0;
  // Tensors that stay unchanged while registered (a solver's integrals and
  // vertex blocks): the contraction engine keeps the digit panels it splits
  // from them, one set per layout, and reuses them instead of permuting and
  // splitting again.  Entries are dropped when their tensor is forgotten.
  struct ConstRange {
    const double *p;
    size_t bytes;
  };
  std::vector<ConstRange> const_tensors;
  struct CachedPanels {
    const double *owner;
    std::shared_ptr<EmuPanels> panels;
    size_t bytes;
  };
  std::map<std::string, CachedPanels> panel_cache;
  size_t panel_cache_bytes = 0;
  bool use_panel_cache = true;
  static constexpr size_t PANEL_CACHE_LIMIT = (size_t)12 << 30;
  void register_constant(const double *p, size_t bytes) {
    if (p && bytes) const_tensors.push_back({p, bytes});
  }
  bool is_constant(const double *p, size_t bytes) const {
    for (const auto &r : const_tensors)
      if (p >= r.p && (const char *)(p) + bytes <= (const char *)(r.p) + r.bytes) return true;
    return false;
  }
  void forget_constant(const double *p) {
    for (size_t i = 0; i < const_tensors.size(); ++i) {
      if (const_tensors[i].p != p) continue;
      const char *lo = (const char *)p, *hi = lo + const_tensors[i].bytes;
      for (auto it = panel_cache.begin(); it != panel_cache.end();) {
        const char *o = (const char *)it->second.owner;
        if (o >= lo && o < hi) {
          panel_cache_bytes -= it->second.bytes;
          it = panel_cache.erase(it);
        } else {
          ++it;
        }
      }
      const_tensors.erase(const_tensors.begin() + i);
      return;
    }
  }
  // Operands unchanged for the length of one residual evaluation (the
  // amplitudes and X = T2 + T1 T1): their digit panels, split once per layout
  // and role, are kept for the evaluation and dropped at its end (so inside a
  // captured iteration they live and die within the graph).
  std::vector<ConstRange> frozen_tensors;
  std::map<std::string, std::shared_ptr<EmuPanels>> frozen_panels;
  size_t frozen_bytes = 0;
  static constexpr size_t FROZEN_PANEL_LIMIT = (size_t)3 << 30;
  void drop_frozen_panels() {
    frozen_panels.clear();
    frozen_bytes = 0;
  }
  bool is_frozen(const double *p, size_t bytes) const {
    for (const auto &r : frozen_tensors)
      if (p >= r.p && (const char *)(p) + bytes <= (const char *)(r.p) + r.bytes) return true;
    return false;
  }
  // injected fault (GBCC_FAULT_*), consumed by the first matching event
  // (never while the stream is being captured into a graph: the fault would
  // be baked into every replay)
  int fault = GBCC_FAULT_NONE;
  bool take_fault(int kind) {
    if (fault != kind) return false;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
      return false;
    fault = GBCC_FAULT_NONE;
    return true;
  }
  // sticky device error word: kernels whose bounded waits give up record a
  // code here; read (and cleared) at synchronisation points
  int *dev_err = nullptr;
  int *device_error_word() {
    if (!dev_err) {
      if (cudaMalloc(&dev_err, sizeof(int)) != cudaSuccess)
        throw Error(GBCC_OOM, "cannot allocate the device error word");
      if (cudaMemsetAsync(dev_err, 0, sizeof(int), stream) != cudaSuccess)
        throw Error(GBCC_CUDA_ERROR, "cannot clear the device error word");
    }
    return dev_err;
  }
  // synchronises the stream; throws GBCC_TIMEOUT if a kernel recorded an error
  void check_device_errors() {
    if (cudaStreamSynchronize(stream) != cudaSuccess)
      throw Error(GBCC_CUDA_ERROR, "stream synchronisation failed");
    if (!dev_err) return;
    int h = 0;
    if (cudaMemcpy(&h, dev_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      throw Error(GBCC_CUDA_ERROR, "cannot read the device error word");
    if (h != 0) {
      cudaMemset(dev_err, 0, sizeof(int));
      throw Error(GBCC_TIMEOUT, "a bounded device wait gave up (code " +
                                    std::to_string(h) + ")");
    }
  }
  // optional per-launch timing of the tensor-core GEMM kernel (CUDA events
  // recorded on the context stream around each launch)
  bool prof = false;
  struct ProfRec {
    cudaEvent_t a, b;
    double tc_flops, fp64_flops;
    int64_t M, N, K;
  };
  struct GemmLog {
    int64_t M, N, K;
    double ms;
  };
  std::vector<ProfRec> prof_recs;
  std::vector<GemmLog> prof_log;  // per launch, until read through the ABI
  std::vector<cudaEvent_t> prof_pool;
  double prof_ms = 0, prof_tc_flops = 0, prof_fp64_flops = 0;
  int64_t prof_launches = 0;
  cudaEvent_t prof_event() {
    if (!prof_pool.empty()) {
      cudaEvent_t e = prof_pool.back();
      prof_pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  void prof_harvest() {
    for (auto &r : prof_recs) {
      cudaEventSynchronize(r.b);
      float ms = 0;
      cudaEventElapsedTime(&ms, r.a, r.b);
      prof_ms += ms;
      if (prof_log.size() < (size_t)1 << 20) prof_log.push_back({r.M, r.N, r.K, (double)ms});
      prof_tc_flops += r.tc_flops;
      prof_fp64_flops += r.fp64_flops;
      prof_launches++;
      prof_pool.push_back(r.a);
      prof_pool.push_back(r.b);
    }
    prof_recs.clear();
  }
};

// Stream-ordered device buffer (cudaMallocAsync on the context stream).
class DBuf {
 public:
  DBuf() = default;
  DBuf(Context &ctx, size_t bytes) { alloc(ctx, bytes); }
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept { *this = std::move(o); }
  DBuf &operator=(DBuf &&o) noexcept {
    if (this != &o) {
      release();
      p_ = o.p_;
      bytes_ = o.bytes_;
      stream_ = o.stream_;
      o.p_ = nullptr;
      o.bytes_ = 0;
    }
    return *this;
  }
  ~DBuf() { release(); }
  void alloc(Context &ctx, size_t bytes) {
    release();
    stream_ = ctx.stream;
    bytes_ = bytes;
    if (bytes == 0) return;
    if (ctx.take_fault(GBCC_FAULT_OOM)) {
      bytes_ = 0;
      throw Error(GBCC_OOM, "injected allocation failure");
    }
    GBCC_CUDA(cudaMallocAsync(&p_, bytes, ctx.stream));
  }
  void release() {
    if (p_) cudaFreeAsync(p_, stream_);
    p_ = nullptr;
    bytes_ = 0;
  }
  template <class T = double>
  T *as() const { return static_cast<T *>(p_); }
  size_t bytes() const { return bytes_; }

 private:
  void *p_ = nullptr;
  size_t bytes_ = 0;
  cudaStream_t stream_ = nullptr;
};

// Dense column-major FP64 tensor view (first index fastest), up to order 6.
struct Ten {
  double *p = nullptr;
  int order = 0;
  std::array<int64_t, 6> lens{};
  int64_t size() const {
    int64_t s = 1;
    for (int d = 0; d < order; ++d) s *= lens[d];
    return s;
  }
};

inline Ten ten(double *p, std::initializer_list<int64_t> l) {
  Ten t;
  t.p = p;
  t.order = static_cast<int>(l.size());
  int d = 0;
  for (auto x : l) t.lens[d++] = x;
  return t;
}
inline Ten ten(double *p, const std::vector<int64_t> &l) {
  require(l.size() <= 6, "tensor order above 6");
  Ten t;
  t.p = p;
  t.order = static_cast<int>(l.size());
  int d = 0;
  for (auto x : l) t.lens[d++] = x;
  return t;
}

// Owned tensor = buffer + view.
// Marks tensors as unchanged until the scope ends (Context::frozen_tensors)
// and drops their kept panels then.
struct FrozenScope {
  Context &ctx;
  explicit FrozenScope(Context &c) : ctx(c) {}
  void add(const double *p, size_t bytes) {
    if (p && bytes) ctx.frozen_tensors.push_back({p, bytes});
  }
  ~FrozenScope() {
    ctx.drop_frozen_panels();
    ctx.frozen_tensors.clear();
  }
  FrozenScope(const FrozenScope &) = delete;
  FrozenScope &operator=(const FrozenScope &) = delete;
};

struct OTen {
  DBuf buf;
  Ten t;
  OTen() = default;
  OTen(Context &ctx, std::initializer_list<int64_t> l) {
    t = ten(nullptr, l);
    buf.alloc(ctx, sizeof(double) * t.size());
    t.p = buf.as<double>();
  }
  OTen(Context &ctx, const std::vector<int64_t> &l) {
    t = ten(nullptr, l);
    buf.alloc(ctx, sizeof(double) * t.size());
    t.p = buf.as<double>();
  }
  operator Ten &() { return t; }
  operator const Ten &() const { return t; }
  double *p() const { return t.p; }
};

// ---------------------------------------------------------------- kernels
// GEMM: C[M,N] = alpha op(A) op(B) + beta C (column-major), batched with
// constant strides.  precision: GBCC_PREC_FP64 or GBCC_PREC_EMU.
void gemm(Context &ctx, bool ta, bool tb, int64_t M, int64_t N, int64_t K,
          double alpha, const double *A, int64_t lda, const double *B,
          int64_t ldb, double beta, double *C, int64_t ldc, int64_t batch = 1,
          int64_t sA = 0, int64_t sB = 0, int64_t sC = 0,
          int precision = GBCC_PREC_FP64);
void gemm_f64(Context &ctx, bool ta, bool tb, int64_t M, int64_t N, int64_t K,
              double alpha, const double *A, int64_t lda, const double *B,
              int64_t ldb, double beta, double *C, int64_t ldc, int64_t batch,
              int64_t sA, int64_t sB, int64_t sC);
// pointer-array batched FP64 GEMM (device arrays of pointers)
void gemm_f64_ptr(Context &ctx, bool ta, bool tb, int64_t M, int64_t N,
                  int64_t K, double alpha, const double *const *A, int64_t lda,
                  const double *const *B, int64_t ldb, double beta,
                  double *const *C, int64_t ldc, int64_t batch);
void gemm_emu(Context &ctx, bool ta, bool tb, int64_t M, int64_t N, int64_t K,
              double alpha, const double *A, int64_t lda, const double *B,
              int64_t ldb, double beta, double *C, int64_t ldc, int64_t batch,
              int64_t sA, int64_t sB, int64_t sC);
// Digit panels of a family of `count` same-shape operands (operand p at
// base + p*pstride, element (r, k) at r*rs + k*ks), split once and reused by
// many emulated GEMMs.  role_a: A operand (rows = M), else B (rows = N).
// Second level of an operand's row and K offsets: with rl > 0, row r sits
// at (r % rl) rs + (r / rl) rs1 (likewise K index k with kl, ks, ks1), so an
// operand whose row (or K) indices form two runs of a tensor is read in
// place; rl = kl = 0 is the plain r rs + k ks.
struct IdxMap {
  unsigned rl = 0, kl = 0;
  int64_t rs1 = 0, ks1 = 0;
};
struct EmuPanels {
  DBuf panels, exps;
  bool role_a = true;
  int S = 6, count = 0, rt = 0, kt = 0;
  int64_t rows = 0, K = 0, rs = 0, ks = 0;
  IdxMap map;
};
EmuPanels emu_split(Context &ctx, bool role_a, const double *base, int64_t R,
                    int64_t K, int64_t rs, int64_t ks, int count, int64_t pstride,
                    const IdxMap &map = IdxMap{});
// C[M,N] = alpha A_ia B_ib^T + beta C with M = A.rows, N = B.rows, K = A.K.
// With Cdf given, C is a float-float array instead (hi and lo rounded from
// the exact fixed-point totals; alpha = +-2^k, beta in {0, 1}).
struct df32;
void emu_gemm_panels(Context &ctx, const EmuPanels &A, int ia, const EmuPanels &B,
                     int ib, double alpha, double beta, double *C, int64_t ldc,
                     df32 *Cdf = nullptr);
// Grouped form: nprob products of the same shape in one launch, problem q
// multiplying operand ia[q] of A with operand ib[q] of B into C[q] (or Cdf[q]).
void emu_gemm_panels_grouped(Context &ctx, const EmuPanels &A, const int *ia,
                             const EmuPanels &B, const int *ib, int nprob, double alpha,
                             double beta, double *const *C, df32 *const *Cdf, int64_t ldc);
// Output index map of an emulated GEMM: C(m, n) at C + (m % ml0) ms0 +
// (m / ml0) ms1 + (n % nl0) ns0 + (n / nl0) ns1 (ml0 = 0: no map).
struct OutMap {
  int64_t ml0, ms0, ms1, nl0, ns0, ns1;
};
// Strided batch: problem q multiplies operand q of A with operand q of B into
// C + q sC (through the output map, if one is given, instead of ldc), in one
// launch that can be captured into a graph.
void emu_gemm_panels_batched(Context &ctx, const EmuPanels &A, const EmuPanels &B, int nprob,
                             double alpha, double beta, double *C, int64_t ldc, int64_t sC,
                             const OutMap &map = OutMap{});
// C = alpha A_ia B_ib^T + beta C written through an output index map.
void emu_gemm_panels_mapped(Context &ctx, const EmuPanels &A, int ia, const EmuPanels &B,
                            int ib, double alpha, double beta, double *C, const OutMap &map);
// Panels of one operand, allocated but not filled (their digits and row
// exponents are written by a producer such as emu_gemm_panels_to_panels).
EmuPanels emu_panels_alloc(Context &ctx, bool role_a, int64_t R, int64_t K);
// The particle ladder's V[(x,c),(d,y)] = sum_G A[G,(x,c)] B[G,(d,y)], from
// the operands' digit panels (A_ia rows m = x + px c, B_ib rows n = d + pd y,
// K = G), written straight into the digit panels P of the next product's A
// operand: rows x + px y, K index d + pd c, with P's row exponents set
// beforehand (ladder_row_exponents).  pd % 8 == 0.  Operands shared by
// several products are split once.
void emu_gemm_panels_to_panels(Context &ctx, const EmuPanels &A, int ia, const EmuPanels &B,
                               int ib, int64_t px, int64_t pd, EmuPanels &P);
// amax[a] = max_c ||dG[., a, c]|| (dG [G, Nv, Nv]); amax holds Nv 64-bit words
void ladder_amax(Context &ctx, const double *dG, int64_t G, int64_t Nv, void *amax);
// er[x + nx y]: exponent bound of V[x0 + x, y0 + y, ., .] from amax (Cauchy-Schwarz)
void ladder_row_exponents(Context &ctx, const void *amax, int64_t x0, int64_t nx, int64_t y0,
                          int64_t ny, int *er);
// Output index map of an emulated GEMM with two indices on each side: C(m, n)
// lives at C + (m % ml0) ms0 + (m / ml0) ms1 + (n % nl0) ns0 + (n / nl0) ns1,
// so a product can write a permuted layout directly (beta must be 0).
void gemm_emu_mapped(Context &ctx, bool ta, bool tb, int64_t M, int64_t N, int64_t K,
                     double alpha, const double *A, int64_t lda, const double *B,
                     int64_t ldb, double *C, const OutMap &map);
// emulated GEMM with its scratch in a fixed file-scope device array
void gemm_emu_noalloc(Context &ctx, bool ta, bool tb, int64_t M, int64_t N,
                      int64_t K, double alpha, const double *A, int64_t lda,
                      const double *B, int64_t ldb, double beta, double *C,
                      int64_t ldc);

// dst[perm-out] = alpha * src + beta * dst, where dst index d of the output
// tensor corresponds to src dimension perm[d]. dst_lens[d] = src.lens[perm[d]].
void permute(Context &ctx, const Ten &src, const int *perm, double alpha,
             double beta, Ten &dst);
void fill(Context &ctx, double *p, int64_t n, double v);
void copy(Context &ctx, double *dst, const double *src, int64_t n);
// y = a*x + b*y  (elementwise, mul-then-add rounding, no FMA)
void axpby(Context &ctx, int64_t n, double a, const double *x, double b,
           double *y);

// ------------------------------------------------------- contraction engine
// C[ic] = alpha * A[ia] B[ib] + beta * C[ic]   (einsum-like on index strings;
// every index of C appears in A or B; summed indices appear in both A and B).
void contract(Context &ctx, double alpha, const Ten &A, const char *ia,
              const Ten &B, const char *ib, double beta, const Ten &C,
              const char *ic, int precision);
// C[ic] = alpha * A[ia] + beta * C[ic]  (pure index permutation)
void assign(Context &ctx, double alpha, const Ten &A, const char *ia,
            double beta, const Ten &C, const char *ic);

}  // namespace gbcc
