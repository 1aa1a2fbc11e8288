// FP64 GEMM emulated on the tcgen05 bf16 tensor cores (sm_103a).
//
//   C = alpha op(A) op(B) + beta C       (column-major FP64 in and out)
//
// Numerics (Ozaki-style fixed-point splitting).  Each row i of op(A) is
// scaled by 2^-ea_i (ea_i = exponent of the row's max |.|) and rounded to an
// integer X with F = 7 S fractional bits, which is then written as S balanced
// base-128 digits d_0 (|d_0| <= 128) ... d_{S-1} (|d| <= 64), so
//   A_ik = 2^ea_i sum_s d_s(i,k) 2^-7(s+1)   (error <= 2^(ea_i - 7S - 1)).
// Columns of op(B) likewise.  Digits are exact in bf16.  The product keeps the
// pairs (s, t) with s + t < S and accumulates every "diagonal" g = s + t in its
// own FP32 TMEM accumulator: digit products and their sums stay integers below
// 2^24 over a K-chunk of 512 (256 for S > 6), so the FP32 sums are exact.
// After each chunk the epilogue warps fold the diagonals into a per-output
// int64 fixed-point total (29 fractional bits below the g = 0 unit), still
// exact up to the rounding of diagonals g >= 5.  At the end the total becomes
// C = 2^(ea_i + eb_j - 14 - 29) * total with integer instructions (one
// rounding, the bits of ldexp((double)total, e)); only a non-zero beta costs
// an FP64 instruction per output.  GB300's FP64 pipe issues a few operations
// per clock per SM, so FP64 work per output would bound the short-K products.
// A float-float output variant (DF) sums the exact FP32 diagonals into hi+lo
// FP32 pairs instead, for consumers that compute in float-float.
//
// Data movement.  A split kernel writes the digits of A (B) as pre-tiled
// operand panels: tiles of 128 (64) rows x 32 k in the no-swizzle K-major
// core-matrix layout (8 rows x 16 B per core matrix, k-groups fastest), one
// contiguous 8 KB (4 KB) block per tile and digit.  The GEMM kernel moves a
// k-block of all S digit tiles of A and B into shared memory with 1-D bulk
// copies (cp.async.bulk, the TMA engine) through a multi-stage mbarrier
// pipeline.  Warp roles: warp 0 producer, warp 1 MMA issuer (one thread,
// tcgen05.mma kind::f16, M=128, K=16, N up to 256: the B digits that pair
// with one A digit are stacked along N), warps 2-17 epilogue (tcgen05.ld).
// The kernel is persistent: one CTA per SM walks its share of the output
// tiles, and the epilogue hands TMEM back to the MMA issuer as soon as it has
// folded a chunk, so the conversion and store of one tile overlap the MMAs
// of the next.  Every wait is bounded; on timeout the kernel records an error
// code, drains what it issued (bounded) and frees its TMEM.
#include <algorithm>
#include <climits>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "df32.hpp"
#include "internal.hpp"

namespace gbcc {
namespace {

constexpr int TM = 128;        // rows of an A tile / CTA tile M
constexpr int TN = 64;         // rows of a B tile / CTA tile N
constexpr int KB = 32;         // k per tile
constexpr int A_TILE = TM * KB * 2;  // bytes
constexpr int B_TILE = TN * KB * 2;
constexpr int FRAC = 29;       // fractional bits of the int64 total (g=0 units)
constexpr int EPI_WARPS = 16;        // epilogue warps (4 per TMEM lane quarter)
constexpr int EPI_COLS = TN / (EPI_WARPS / 4);  // output columns per epilogue thread
constexpr int NUM_THREADS = 64 + 32 * EPI_WARPS;
constexpr int SMEM_BUDGET = 220 * 1024;
constexpr long long WAIT_LIMIT = 1LL << 26;
constexpr int GROUP_M = 16;    // m-tiles per rasterization group
// exponents start at a large negative sentinel (all-zero rows keep it); any
// value below EXP_FLOOR means "row is zero"
constexpr int EXP_FLOOR = -1100;

enum : int { ERR_NONE = 0, ERR_FULL = 1, ERR_EMPTY = 2, ERR_ACCF = 3,
             ERR_ACCE = 4, ERR_DRAIN = 5, ERR_INJECTED = 6 };
// polls of the injected wait (a barrier nothing completes): well under a second
constexpr long long INJECTED_WAIT_LIMIT = 1LL << 16;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait: false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long i = 0; i < WAIT_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// bounded wait that also gives up as soon as another role of the CTA has
// aborted (checked every 64 polls), so that one failure ends the kernel
// promptly instead of running every other wait to its limit
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t bar, uint32_t parity,
                                                   const volatile int *abort,
                                                   long long limit = WAIT_LIMIT) {
  for (long long i = 0; i < limit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63) == 63 && *abort) return false;
  }
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src,
                                         uint32_t bytes, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

// no-swizzle K-major shared-memory matrix descriptor (tcgen05 format):
// [0,14) start>>4, [16,30) LBO>>4 (K-adjacent core matrices),
// [32,46) SBO>>4 (M/N-adjacent core matrices), [46,48) version = 1,
// [61,64) layout = 0 (no swizzle)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo,
                                              uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t a, uint64_t b,
                                         uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          bar)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
        "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]),
        "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// Output scaling alpha: (-1)^neg 2^shift when pow2, else a general multiplier.
struct OutScale {
  double alpha;
  int pow2, shift, neg;
};

OutScale out_scale(double alpha) {
  OutScale o{alpha, 0, 0, 0};
  int x = 0;
  const double m = std::frexp(alpha, &x);
  if (m == 0.5 || m == -0.5) {
    o.pow2 = 1;
    o.shift = x - 1;
    o.neg = alpha < 0.0 ? 1 : 0;
  }
  return o;
}

// rare route of fixed_to_double (subnormal or overflowing results)
__device__ __noinline__ double fixed_to_double_slow(long long t, int e) {
  return ldexp(__ll2double_rn(t), e);
}

// t * 2^e rounded once to the nearest double (ties to even): the value of
// ldexp((double)t, e) whenever the result is a normal number, built with
// integer instructions only (leading-zero count, 53-bit round, exponent
// field), because the FP64 pipe of this GPU issues a few instructions per
// clock per SM and the GEMM epilogue converts every output element.
// Subnormal or overflowing results take the FP64 route.
__device__ __forceinline__ double fixed_to_double(long long t, int e) {
  if (t == 0) return 0.0;
  const unsigned long long sgn = (unsigned long long)t & 0x8000000000000000ull;
  unsigned long long mag = t < 0 ? 0ull - (unsigned long long)t : (unsigned long long)t;
  const int lz = __clzll((long long)mag);
  mag <<= lz;                                // leading one at bit 63
  unsigned long long mant = mag >> 11;       // 53 significant bits
  const unsigned rem = (unsigned)(mag & 0x7FFull);
  mant += (rem > 0x400u || (rem == 0x400u && (mant & 1ull))) ? 1ull : 0ull;
  int be = 63 - lz + e + 1023;               // biased exponent of the leading one
  if (mant >> 53) {
    mant >>= 1;
    ++be;
  }
  if (be <= 0 || be >= 2047) return fixed_to_double_slow(t, e);
  return __longlong_as_double(
      (long long)(sgn | ((unsigned long long)be << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// alpha * t * 2^e; a power-of-two alpha costs no FP64 instruction
__device__ __forceinline__ double scaled_total(long long t, int e, const OutScale &o) {
  if (o.pow2) return fixed_to_double(o.neg ? -t : t, e + o.shift);
  return fixed_to_double(t, e) * o.alpha;
}

// bf16 bits of a small integer v (|v| <= 2^8: exact in bf16), FP32-pipe
// and integer instructions only: the magic-number add makes the float v
// exactly, and its upper 16 bits are the bf16 encoding.
__device__ __forceinline__ uint32_t small_int_bf16_bits(int v) {
  const float f = __int_as_float(0x4B400000 + v) - 12582912.0f;  // 1.5 * 2^23
  return __float_as_uint(f) >> 16;
}

// One problem of a grouped launch: many GEMMs of the same M, N, K whose
// operands are panels of the same families (different operand indices) and
// whose outputs are different arrays.
struct EmuProb {
  const __nv_bfloat16 *A, *B;
  const int *ea, *eb;
  double *C;
  df32 *Cdf;
};

struct EmuArgs {
  const __nv_bfloat16 *A;  // [S][mt][kt] tiles
  const __nv_bfloat16 *B;  // [S][nt][kt] tiles
  const int *ea, *eb;      // row / column exponents
  double *C;
  df32 *Cdf;               // float-float output instead of C when not null
  int64_t M, N, ldc;
  int mt, nt, kt;          // tile counts
  int kc_blocks;           // k-blocks per exact chunk
  int kb_per_split;        // k-blocks per K-split (a multiple of kc_blocks)
  int ksplit;              // number of K-splits (1: write C directly)
  int frac;                // fractional bits of the int64 totals
  long long *W;            // K-split totals [ksplit][N][M] (ksplit > 1)
  OutScale os;             // alpha
  double beta;
  int *err;
  // test hook: the MMA issuer first waits on a barrier that nothing
  // completes, so the bounded wait gives up (GBCC_FAULT_DEVICE_WAIT)
  int inject_wait;
  // output index map (OutMap); mapped = 0: C(m, n) at C + m + n ldc
  int mapped;
  unsigned ml0, nl0;
  int64_t ms0, ms1, ns0, ns1;
  // grouped launch: nprob problems of this shape, one table entry each (the
  // pointers above are then unused); nprob = 1 with probs = nullptr is the
  // plain GEMM.  Grouped launches have ksplit = 1.
  int nprob = 1;
  const EmuProb *probs = nullptr;
  // strided batch (probs = nullptr, nprob > 1): problem q uses the operands
  // and output above advanced by q times these element strides
  int64_t qsA = 0, qsB = 0, qsea = 0, qseb = 0, qsC = 0;
  // digit-panel output (the particle ladder): instead of C, the product
  // V[(x,c),(d,y)] is written as the S bf16 digits of the A operand of the
  // next product, rows r = x + px*y, K index k = d + pd*c (m = x + px*c,
  // n = d + pd*y), with the row exponents pexp[r] given (max|V| < 2^pexp[r]);
  // tiles [S][prt][pkt] of TM rows x KB k as split_kernel writes them.
  // Needs beta = 0, ksplit = 1, pd a multiple of 8.
  __nv_bfloat16 *pout = nullptr;
  const int *pexp = nullptr;
  int prt = 0, pkt = 0;
  unsigned px = 0, pd = 0;
  int64_t pplane = 0;
};

// pointers of problem q (the plain GEMM's own for a single problem)
__device__ __forceinline__ EmuProb problem_of(const EmuArgs &a, int q) {
  if (a.probs) return a.probs[q];
  EmuProb p;
  p.A = a.A + q * a.qsA;
  p.B = a.B + q * a.qsB;
  p.ea = a.ea + q * a.qsea;
  p.eb = a.eb + q * a.qseb;
  p.C = a.C ? a.C + q * a.qsC : nullptr;
  p.Cdf = a.Cdf ? a.Cdf + q * a.qsC : nullptr;
  return p;
}

// work unit u (a K-split of one output tile) -> split index and tile.
// Grouped rasterization: consecutive units walk GROUP_M m-tiles down one
// column of n-tiles, so that the CTAs working at the same time share a
// compact set of A and B panels in L2.
// (32-bit arithmetic: the host keeps mt * nt * ksplit below 2^31; 64-bit
// integer division would cost FP64-pipe instructions on this GPU)
__device__ __forceinline__ void unit_coords(const EmuArgs &a, int u, int &split,
                                            int &tile_m, int &tile_n) {
  const int ntiles = a.mt * a.nt;
  split = u / ntiles;  // the problem index instead in a grouped launch
  const int t = u - split * ntiles;
  const int gsz = GROUP_M * a.nt;
  const int g = t / gsz, r = t - g * gsz;
  const int first = g * GROUP_M;
  const int gm = min(GROUP_M, a.mt - first);
  tile_m = first + r % gm;
  tile_n = r / gm;
}

// a * 2^k for a float-float a (exact unless the result leaves the FP32 range)
__device__ __forceinline__ df32 df_ldexp(df32 v, int k) {
  while (k > 127 || k < -126) {
    const int step = k > 0 ? 127 : -126;
    const float f = __int_as_float((step + 127) << 23);
    v = df_make(v.hi * f, v.lo * f);
    k -= step;
    if (v.hi == 0.0f) return v;
  }
  const float f = __int_as_float((k + 127) << 23);
  return df_make(v.hi * f, v.lo * f);
}

// a + b for an FP32 b (TwoSum of the leading parts, then Fast2Sum)
__device__ __forceinline__ df32 df_add_f(df32 a, float b) {
  const float s = a.hi + b;
  const float bb = s - a.hi;
  const float e = ((a.hi - (s - bb)) + (b - bb)) + a.lo;
  return df_fast2sum(s, e);
}

// DF: float-float output (a.Cdf).  The exact FP32 diagonal sums are then
// added straight into a float-float accumulator, smallest diagonal first, on
// the FP32 pipe; otherwise they fold into an exact int64 total.
template <int S, bool DF>
__global__ void __launch_bounds__(NUM_THREADS, 1) emu_gemm_kernel(EmuArgs a) {
  constexpr int STAGE_BYTES = S * (A_TILE + B_TILE);
  constexpr int STAGES = (SMEM_BUDGET / STAGE_BYTES) > 4 ? 4 : (SMEM_BUDGET / STAGE_BYTES);
  static_assert(STAGES >= 2, "not enough shared memory for two stages");
  constexpr uint32_t TMEM_COLS = (S * TN <= 256) ? 256 : 512;
  static_assert(S * TN <= 512, "too many diagonals for TMEM");

  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar_full[4], bar_empty[4], bar_accf, bar_acce,
      bar_drain, bar_never;
  __shared__ uint32_t tmem_base_sh;
  __shared__ volatile int abort_sh;

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int nunits = a.mt * a.nt * a.ksplit * a.nprob;
  const bool grouped = a.nprob > 1;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&bar_full[s]), 1);
      mbar_init(smem_u32(&bar_empty[s]), 1);
    }
    mbar_init(smem_u32(&bar_accf), 1);
    mbar_init(smem_u32(&bar_acce), 32 * EPI_WARPS);
    mbar_init(smem_u32(&bar_drain), 1);
    mbar_init(smem_u32(&bar_never), 1);
    abort_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
            smem_u32(&tmem_base_sh)),
        "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;
  const uint32_t smem_base = smem_u32(smem);

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      const size_t a_slice = (size_t)a.mt * a.kt * (A_TILE / 2);
      const size_t b_slice = (size_t)a.nt * a.kt * (B_TILE / 2);
      long long g = 0;  // k-blocks issued by this CTA
      bool ok = true;
      for (int u = blockIdx.x; u < nunits && ok; u += gridDim.x) {
        int split, tile_m, tile_n;
        unit_coords(a, u, split, tile_m, tile_n);
        const EmuProb pr = problem_of(a, grouped ? split : 0);
        if (grouped) split = 0;
        const int kb0 = split * a.kb_per_split;
        const int nkb = max(0, min(a.kt, kb0 + a.kb_per_split) - kb0);
        for (int kl = 0; kl < nkb; ++kl) {
          const int st = (int)(g % STAGES);
          if (g >= STAGES &&
              !mbar_wait_or_abort(smem_u32(&bar_empty[st]), (int)((g / STAGES) - 1) & 1,
                                  &abort_sh)) {
            atomicCAS(a.err, 0, ERR_EMPTY);
            abort_sh = 1;
            ok = false;
            break;
          }
          if (abort_sh) {
            ok = false;
            break;
          }
          const int kb = kb0 + kl;
          const uint32_t full = smem_u32(&bar_full[st]);
          mbar_expect_tx(full, STAGE_BYTES);
          const uint32_t sbase = smem_base + st * STAGE_BYTES;
          for (int s = 0; s < S; ++s) {
            const __nv_bfloat16 *ga =
                pr.A + s * a_slice + ((size_t)tile_m * a.kt + kb) * (A_TILE / 2);
            bulk_g2s(sbase + s * A_TILE, ga, A_TILE, full);
          }
          for (int s = 0; s < S; ++s) {
            const __nv_bfloat16 *gb =
                pr.B + s * b_slice + ((size_t)tile_n * a.kt + kb) * (B_TILE / 2);
            bulk_g2s(sbase + S * A_TILE + s * B_TILE, gb, B_TILE, full);
          }
          ++g;
        }
      }
      // never leave a bulk copy in flight: wait (bounded) for the last
      // STAGES issued k-blocks to land
      for (long long k = g > STAGES ? g - STAGES : 0; k < g; ++k)
        mbar_wait(smem_u32(&bar_full[k % STAGES]), (int)(k / STAGES) & 1);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      long long g = 0;   // k-blocks consumed
      long long cg = 0;  // chunks issued
      bool ok = true;
      if (a.inject_wait &&
          !mbar_wait_or_abort(smem_u32(&bar_never), 0, &abort_sh, INJECTED_WAIT_LIMIT)) {
        atomicCAS(a.err, 0, ERR_INJECTED);
        abort_sh = 1;
        ok = false;
      }
      for (int u = blockIdx.x; u < nunits && ok; u += gridDim.x) {
        int split, tile_m, tile_n;
        unit_coords(a, u, split, tile_m, tile_n);
        if (grouped) split = 0;
        const int kb0 = split * a.kb_per_split;
        const int nkb = max(0, min(a.kt, kb0 + a.kb_per_split) - kb0);
        const int nchunks = (nkb + a.kc_blocks - 1) / a.kc_blocks;
        int kl = 0;
        for (int c = 0; c < nchunks; ++c) {
          // TMEM is free once the epilogue has folded the previous chunk
          if (cg > 0 && !mbar_wait_or_abort(smem_u32(&bar_acce), (int)(cg - 1) & 1, &abort_sh)) {
            atomicCAS(a.err, 0, ERR_ACCE);
            abort_sh = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          const int kend = min(nkb, (c + 1) * a.kc_blocks);
          const int kfirst = kl;
          for (; kl < kend; ++kl) {
            const int st = (int)(g % STAGES);
            if (!mbar_wait_or_abort(smem_u32(&bar_full[st]), (int)(g / STAGES) & 1, &abort_sh)) {
              atomicCAS(a.err, 0, ERR_FULL);
              abort_sh = 1;
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sbase = smem_base + st * STAGE_BYTES;
            // Pairs (s, t) go to diagonal g = s + t at TMEM columns g*TN, so
            // all pairs of one A digit s write the contiguous column range
            // [s*TN, S*TN): one MMA per s (split at N = 256) whose B operand is
            // the B digit tiles t = 0..S-1-s stacked along N (consecutive 4 KB
            // tiles keep the 512 B row-group stride).  The first MMA of a chunk
            // (s = 0, k16 = 0) overwrites every diagonal.
#pragma unroll
            for (int k16 = 0; k16 < KB / 16; ++k16) {
#pragma unroll
              for (int s = 0; s < S; ++s) {
                const uint64_t da = smem_desc(sbase + s * A_TILE + k16 * 256, 128,
                                              (KB / 8) * 128);
                const uint32_t acc = (kl == kfirst && k16 == 0 && s == 0) ? 0u : 1u;
#pragma unroll
                for (int off = 0; off < (S - s) * TN; off += 256) {
                  const int n = min(256, (S - s) * TN - off);
                  const uint64_t db =
                      smem_desc(sbase + S * A_TILE + (off / TN) * B_TILE + k16 * 256,
                                128, (KB / 8) * 128);
                  mma_bf16(tmem + s * TN + off, da, db, instr_desc(TM, n), acc);
                }
              }
            }
            mma_commit(smem_u32(&bar_empty[st]));
            ++g;
          }
          if (!ok) break;
          mma_commit(smem_u32(&bar_accf));
          ++cg;
        }
      }
      // make sure every issued MMA finished before TMEM is released
      mma_commit(smem_u32(&bar_drain));
      if (!mbar_wait(smem_u32(&bar_drain), 0)) atomicCAS(a.err, 0, ERR_DRAIN);
      if (!ok) abort_sh = 1;
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ epilogue
    const int ew = warp - 2;             // 0..EPI_WARPS-1
    const int quarter = warp & 3;        // TMEM lane quarter this warp may access
    const int cgrp = ew >> 2;            // column group of EPI_COLS columns
    const int row = quarter * 32 + lane; // row within the tile
    const uint32_t lane_addr = tmem + ((uint32_t)(quarter * 32) << 16);
    long long cg = 0;  // chunks consumed
    for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
      int split, tile_m, tile_n;
      unit_coords(a, u, split, tile_m, tile_n);
      const EmuProb pr = problem_of(a, grouped ? split : 0);
      if (grouped) split = 0;
      const int kb0 = split * a.kb_per_split;
      const int nkb = max(0, min(a.kt, kb0 + a.kb_per_split) - kb0);
      const int nchunks = (nkb + a.kc_blocks - 1) / a.kc_blocks;
      long long tot[DF ? 1 : EPI_COLS];
      df32 acc[DF ? EPI_COLS : 1];
#pragma unroll
      for (int j = 0; j < (DF ? 1 : EPI_COLS); ++j) tot[j] = 0;
#pragma unroll
      for (int j = 0; j < (DF ? EPI_COLS : 1); ++j) acc[j] = df_make(0.0f, 0.0f);
      bool ok = true;
      for (int c = 0; c < nchunks; ++c) {
        if (!mbar_wait_or_abort(smem_u32(&bar_accf), (int)(cg & 1), &abort_sh)) {
          atomicCAS(a.err, 0, ERR_ACCF);
          abort_sh = 1;
          ok = false;
          break;
        }
        if (abort_sh) {
          ok = false;
          break;
        }
        tc_fence_after();
        if constexpr (DF) {
          // acc += sum_g x_g 2^(-7g), units of the g = 0 digit product
#pragma unroll
          for (int g = S - 1; g >= 0; --g) {
            const float w = __int_as_float((127 - 7 * g) << 23);  // 2^(-7g), exact scaling
            float v[16];
            tmem_ld16(lane_addr + g * TN + cgrp * EPI_COLS, v);
#pragma unroll
            for (int j = 0; j < EPI_COLS; ++j) acc[j] = df_add_f(acc[j], v[j] * w);
          }
        } else {
#pragma unroll
          for (int g = 0; g < S; ++g) {
            const int sh = a.frac - 7 * g;
            float v[16];
            tmem_ld16(lane_addr + g * TN + cgrp * EPI_COLS, v);
#pragma unroll
            for (int j = 0; j < EPI_COLS; ++j) {
              const long long x = (long long)__float2int_rn(v[j]);  // exact, |v| <= 2^24
              long long y;
              if (sh >= 0) y = x << sh;
              else y = (x + (1LL << (-sh - 1))) >> (-sh);
              tot[j] += y;
            }
          }
        }
        tc_fence_before();
        mbar_arrive(smem_u32(&bar_acce));
        ++cg;
      }
      if (!ok || abort_sh) break;
      // write out: C[m + n ldc], m = tile_m*128 + row, n = n0 + j.  The column
      // exponents are loaded once (one per lane) and broadcast by shuffles,
      // and C is read in batches of 8 columns, so the write-out waits on a
      // few memory latencies instead of one per column.
      const int64_t m = (int64_t)tile_m * TM + row;
      const int64_t n0 = (int64_t)tile_n * TN + cgrp * EPI_COLS;
      if (a.ksplit == 1) {
        const int ebl =
            (lane < EPI_COLS && n0 + lane < a.N) ? max(pr.eb[n0 + lane], EXP_FLOOR) : 0;
        const bool mrow = m < a.M;
        const int ea = mrow ? max(pr.ea[m], EXP_FLOOR) - 14 - a.frac : 0;
        const bool accumulate = a.beta != 0.0;
        if constexpr (DF) {
          // float-float output; alpha = +-2^k and beta in {0, 1} (host-checked)
          const int ea_df = mrow ? max(pr.ea[m], EXP_FLOOR) - 14 + a.os.shift : 0;
          df32 *cp = pr.Cdf + m + n0 * a.ldc;
#pragma unroll
          for (int j0 = 0; j0 < EPI_COLS; j0 += 8) {
            df32 c[8];
#pragma unroll
            for (int j = 0; j < 8; ++j)
              c[j] = (accumulate && mrow && n0 + j0 + j < a.N) ? cp[(j0 + j) * a.ldc]
                                                              : df_make(0.0f, 0.0f);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const int eb = __shfl_sync(0xffffffffu, ebl, j0 + j);
              if (!mrow || n0 + j0 + j >= a.N) continue;
              df32 v = df_ldexp(acc[j0 + j], ea_df + eb);
              if (a.os.neg) v = df_neg(v);
              if (accumulate) v = df_add(v, c[j]);
              cp[(j0 + j) * a.ldc] = v;
            }
          }
        } else {
        if (a.pout) {
          // digit-panel output: each 8-column half of this thread's 16
          // columns holds 8 consecutive d of one y (pd is a multiple of 8),
          // so each digit of a half is one 16-byte row segment of a panel tile
          // (n0 is the same for the whole warp; rows past M only skip their
          // stores, so that every lane takes part in the shuffles below)
          if (n0 >= a.N) continue;
          const unsigned mu = mrow ? (unsigned)m : 0u;
          const unsigned x = mu % a.px, c = mu / a.px;
          const int F = 7 * S;
          long long bias = 0;
#pragma unroll
          for (int q = 1; q < S; ++q) bias += 64LL << (7 * (S - 1 - q));
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const unsigned nu = (unsigned)n0 + 8u * h;
            if (nu >= (unsigned)a.N) break;  // warp-uniform
            const unsigned d0 = nu % a.pd, y = nu / a.pd;
            const unsigned r = x + a.px * y;
            const unsigned k0 = d0 + a.pd * c;
            const int er = mrow ? a.pexp[r] : EXP_FLOOR - 1;
            const unsigned rr = r % TM, tr = r / TM;
            const unsigned tk = k0 / KB, kk = k0 % KB;  // kk is a multiple of 8
            const int64_t off = ((int64_t)tr * a.pkt + tk) * (TM * KB) +
                                (int64_t)(((rr / 8) * (KB / 8) + kk / 8) * 64 + (rr % 8) * 8);
            uint32_t packed[S][4];
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) {
              const int j = 8 * h + jj;
              const int eb = __shfl_sync(0xffffffffu, ebl, j);
              const long long t = tot[j];
              long long X = 0;
              if (t != 0 && er >= EXP_FLOOR) {
                const int sh = ea + eb + F - er;
                const unsigned long long mag =
                    t < 0 ? 0ull - (unsigned long long)t : (unsigned long long)t;
                unsigned long long xm;
                if (sh >= 0) xm = sh > 62 ? 0ull : (mag << sh);
                else if (sh <= -63) xm = 0ull;
                else xm = (mag + (1ull << (-sh - 1))) >> (-sh);
                X = t < 0 ? -(long long)xm : (long long)xm;
              }
              const long long Y = X + bias;
#pragma unroll
              for (int q = 0; q < S; ++q) {
                const int dg = q == 0 ? (int)(Y >> (7 * (S - 1)))
                                      : (int)((Y >> (7 * (S - 1 - q))) & 127) - 64;
                const uint32_t bits = small_int_bf16_bits(dg);
                if (jj % 2 == 0) packed[q][jj / 2] = bits;
                else packed[q][jj / 2] |= bits << 16;
              }
            }
            if (mrow) {
#pragma unroll
              for (int q = 0; q < S; ++q)
                *reinterpret_cast<uint4 *>(a.pout + q * a.pplane + off) =
                    make_uint4(packed[q][0], packed[q][1], packed[q][2], packed[q][3]);
            }
          }
          continue;
        }
        if (a.mapped) {
          // permuted output layout: row offset once, column offsets stepped
          // through the mixed radix of n; every lane runs the same loop (the
          // shuffles stay converged); with beta, each output is read where it
          // is written
          const unsigned mu = mrow ? (unsigned)m : 0u;
          const unsigned mq = mu / a.ml0;
          double *rp = pr.C + (int64_t)(mu - mq * a.ml0) * a.ms0 + (int64_t)mq * a.ms1;
          unsigned nq = (unsigned)n0 / a.nl0, nr = (unsigned)n0 - nq * a.nl0;
#pragma unroll
          for (int j = 0; j < EPI_COLS; ++j) {
            const int eb = __shfl_sync(0xffffffffu, ebl, j);
            if (mrow && n0 + j < a.N) {
              double *q = rp + (int64_t)nr * a.ns0 + (int64_t)nq * a.ns1;
              double v = scaled_total(tot[j], ea + eb, a.os);
              if (accumulate) v = fma(a.beta, *q, v);
              *q = v;
            }
            if (++nr == a.nl0) {
              nr = 0;
              ++nq;
            }
          }
          continue;
        }
        double *cp = pr.C + m + n0 * a.ldc;
#pragma unroll
        for (int j0 = 0; j0 < EPI_COLS; j0 += 8) {
          double c[8];
#pragma unroll
          for (int j = 0; j < 8; ++j)
            c[j] = (accumulate && mrow && n0 + j0 + j < a.N) ? cp[(j0 + j) * a.ldc] : 0.0;
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int eb = __shfl_sync(0xffffffffu, ebl, j0 + j);
            if (!mrow || n0 + j0 + j >= a.N) continue;
            double v = scaled_total(tot[j0 + j], ea + eb, a.os);
            if (accumulate) v = fma(a.beta, c[j], v);
            cp[(j0 + j) * a.ldc] = v;
          }
        }
        }
      } else if (m < a.M) {
        // exact partial totals; emu_splitk_reduce adds them in split order
        if constexpr (!DF) {
          long long *w = a.W + (size_t)split * a.N * a.M + m;
#pragma unroll
          for (int j = 0; j < EPI_COLS; ++j) {
            const int64_t n = n0 + j;
            if (n < a.N) w[n * a.M] = tot[j];
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS));
  }
}

// ---------------------------------------------------------------- splitting
// exponent e with max|x| < 2^e over one row (rows of op(A) / columns of op(B)).
// Element (r, k) of the operand lives at base[r*rs + k*ks].
// The row exponent is the largest frexp exponent over the row, so it is a
// max of integers read from the IEEE exponent field: blocks over (rows,
// K-chunks) combine with atomicMax, which is order-independent and therefore
// deterministic.  e[] starts at a large negative sentinel (memset 0x80);
// all-zero rows keep it.
__device__ __forceinline__ int frexp_exponent(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((b >> 52) & 0x7FF);
  return E == 0 ? INT_MIN : E - 1022;  // zero / subnormal: no contribution
}

// row index contiguous (rs == 1): one thread per row, one K-chunk per blockIdx.y
// offset of index v along one operand dimension: v s0, or with a second
// level (l > 0) (v % l) s0 + (v / l) s1 (32-bit division: the host keeps
// mapped dimensions below 2^31)
__device__ __forceinline__ int64_t map_off(int64_t v, int64_t s0, unsigned l, int64_t s1) {
  if (l == 0) return v * s0;
  const unsigned u = (unsigned)v, q = u / l;
  return (int64_t)(u - q * l) * s0 + (int64_t)q * s1;
}

// rows contiguous (rs = 1 at the first level): one thread per row
__global__ void exponent_rows_contig_kernel(const double *__restrict__ base,
                                            int64_t R, int64_t K, int64_t ks,
                                            int64_t kchunk, int *__restrict__ e,
                                            IdxMap mp) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const int64_t k0 = (int64_t)blockIdx.y * kchunk;
  const int64_t k1 = min(K, k0 + kchunk);
  const double *row = base + map_off(r, 1, mp.rl, mp.rs1);
  int m = INT_MIN;
  for (int64_t k = k0; k < k1; ++k) m = max(m, frexp_exponent(row[map_off(k, ks, mp.kl, mp.ks1)]));
  if (m != INT_MIN) atomicMax(&e[r], m);
}

// any strides: one warp per row, one K-chunk per blockIdx.y
__global__ void exponent_rows_warp_kernel(const double *__restrict__ base,
                                          int64_t R, int64_t K, int64_t rs,
                                          int64_t ks, int64_t kchunk,
                                          int *__restrict__ e, IdxMap mp) {
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (r >= R) return;
  const int lane = threadIdx.x % 32;
  const int64_t k0 = (int64_t)blockIdx.y * kchunk;
  const int64_t k1 = min(K, k0 + kchunk);
  const double *row = base + map_off(r, rs, mp.rl, mp.rs1);
  int m = INT_MIN;
  for (int64_t k = k0 + lane; k < k1; k += 32)
    m = max(m, frexp_exponent(row[map_off(k, ks, mp.kl, mp.ks1)]));
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0 && m != INT_MIN) atomicMax(&e[r], m);
}

// fixed-point integer X = round(x 2^(F - e)) from the IEEE bits (integer ops)
__device__ __forceinline__ long long to_fixed(double x, int e, int F) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((bits >> 52) & 0x7FF);
  if (ex == 0) return 0;  // zero or subnormal (below any scale used here)
  const long long mant = (long long)((bits & ((1ULL << 52) - 1)) | (1ULL << 52));
  const int sh = ex - 1075 + F - e;  // x = mant 2^(ex-1075)
  long long X;
  if (sh >= 0) X = mant << sh;       // sh <= 10 since |x| < 2^e
  else if (sh <= -63) X = 0;
  else X = (mant + (1LL << (-sh - 1))) >> (-sh);
  return (bits >> 63) ? -X : X;
}


// digits of one operand into tiles [S][rt][kt] of TR rows x 32 k.
// One thread writes one 16-byte core-matrix row (8 consecutive k) per digit.
// The balanced digits come straight from Y = X + B, B = sum_{s>=1} 64 *
// 128^(S-1-s): d_s = ((Y >> 7(S-1-s)) & 127) - 64 for s >= 1 and
// d_0 = Y >> 7(S-1), the unique representation with d_s in [-64, 63].
// Index arithmetic is 32-bit (the host checks the segment count).
template <int S, int TR>
__global__ void split_kernel(const double *__restrict__ base, int64_t R,
                             int64_t K, int64_t rs, int64_t ks,
                             const int *__restrict__ e, int rt, int kt,
                             __nv_bfloat16 *__restrict__ out, IdxMap mp) {
  const unsigned rows = (unsigned)rt * TR;
  const unsigned segs = rows * (unsigned)kt * (KB / 8);  // 16-byte segments per digit
  constexpr unsigned tile_elems = TR * KB;
  const int64_t plane = (int64_t)rt * kt * tile_elems;
  long long bias = 0;
#pragma unroll
  for (int s = 1; s < S; ++s) bias += 64LL << (7 * (S - 1 - s));
  for (unsigned idx = blockIdx.x * blockDim.x + threadIdx.x; idx < segs;
       idx += gridDim.x * blockDim.x) {
    // idx -> (row r in [0, rt*TR), k-group kg in [0, kt*4)) with r fastest
    const unsigned kg = idx / rows, r = idx - kg * rows;
    const unsigned tr = r / TR, rr = r % TR;
    const unsigned tk = kg / (KB / 8), kk = kg % (KB / 8);
    // destination offset (elements) inside the digit plane
    const int64_t off = ((int64_t)tr * kt + tk) * tile_elems +
                        ((rr / 8) * (KB / 8) + kk) * 64 + (rr % 8) * 8;
    const int er = (r < R) ? e[r] : EXP_FLOOR - 1;
    const bool live = r < R && er >= EXP_FLOOR;  // rows below the floor are all zero
    const double *row = base + (live ? map_off(r, rs, mp.rl, mp.rs1) : 0);
    uint32_t packed[S][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int64_t k = (int64_t)kg * 8 + j;
      long long X = 0;
      if (live && k < K) X = to_fixed(row[map_off(k, ks, mp.kl, mp.ks1)], er, 7 * S);
      const long long Y = X + bias;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int d = s == 0 ? (int)(Y >> (7 * (S - 1)))
                             : (int)((Y >> (7 * (S - 1 - s))) & 127) - 64;
        const uint32_t bits = small_int_bf16_bits(d);
        if (j % 2 == 0) packed[s][j / 2] = bits;
        else packed[s][j / 2] |= bits << 16;
      }
    }
#pragma unroll
    for (int s = 0; s < S; ++s)
      *reinterpret_cast<uint4 *>(out + s * plane + off) =
          make_uint4(packed[s][0], packed[s][1], packed[s][2], packed[s][3]);
  }
}

// Row-exponent bound of the ladder's V blocks.  amax[a] = max_c ||dG[., a, c]||
// over the columns of the dressed vertex dG [G, Nv, Nv] (G fastest), one warp
// per (a, c); the maximum is taken on the IEEE bits of the non-negative
// norms (their integer order), so it does not depend on the order.
__global__ void column_norm_max_kernel(const double *__restrict__ dG, int64_t G,
                                       int64_t ncol, int64_t Nv,
                                       unsigned long long *__restrict__ amax) {
  const int64_t col = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x % 32;
  if (col >= ncol) return;
  const double *p = dG + col * G;
  double s = 0.0;
  for (int64_t g = lane; g < G; g += 32) s = fma(p[g], p[g], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0)
    atomicMax(&amax[col % Nv], (unsigned long long)__double_as_longlong(sqrt(s)));
}

// er[x + nx y] = exponent e with amax[x0 + x] amax[y0 + y] (1 + 2^-20) < 2^e:
// by Cauchy-Schwarz |V[x,y,c,d]| = |sum_G dG[G,x,c] dG[G,y,d]| is below it (the
// factor covers the rounding of the norms and of the operands' digits).  A
// zero bound keeps the "zero row" sentinel.
__global__ void ladder_row_exponent_kernel(const unsigned long long *__restrict__ amax,
                                           int64_t x0, int64_t nx, int64_t y0, int64_t ny,
                                           int *__restrict__ er) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nx * ny) return;
  const int64_t x = r % nx, y = r / nx;
  const double b = __longlong_as_double((long long)amax[x0 + x]) *
                   __longlong_as_double((long long)amax[y0 + y]) * (1.0 + 0x1p-20);
  const int e = frexp_exponent(b);
  er[r] = e == INT_MIN ? (int)0x80808080 : e;
}

// Rows R .. rt*TM of A-role panels (the padding of the last tile row) set to
// the digits of zero, which the panel-output GEMM never writes: one 16-byte
// row segment per thread.
__global__ void zero_panel_rows_kernel(__nv_bfloat16 *__restrict__ P, int64_t R, int rt,
                                       int kt, int S, int64_t plane) {
  const int64_t pad = (int64_t)rt * TM - R;
  const int64_t n = pad * kt * (KB / 8) * S;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t t = i;
    const int64_t row = R + t % pad;
    t /= pad;
    const int seg = (int)(t % (KB / 8));
    t /= (KB / 8);
    const int64_t tk = t % kt;
    const int64_t q = t / kt;
    const int64_t tr = row / TM, rr = row % TM;
    const int64_t off = q * plane + (tr * kt + tk) * (TM * KB) +
                        ((rr / 8) * (KB / 8) + seg) * 64 + (rr % 8) * 8;
    *reinterpret_cast<uint4 *>(P + off) = make_uint4(0u, 0u, 0u, 0u);
  }
}

// out = alpha * 2^(ea+eb-14-frac) * sum_s W[s] + beta * C, summing the exact
// int64 split totals in split order (deterministic)
__global__ void emu_splitk_reduce_kernel(const long long *__restrict__ W, int ks,
                                         int64_t M, int64_t N,
                                         const int *__restrict__ ea,
                                         const int *__restrict__ eb, int frac,
                                         OutScale os, double beta,
                                         double *__restrict__ C, int64_t ldc,
                                         OutMap map) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < M * N;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = i % M, n = i / M;
    long long t = 0;
    for (int s = 0; s < ks; ++s) t += W[((int64_t)s * N + n) * M + m];
    const int e = max(ea[m], EXP_FLOOR) + max(eb[n], EXP_FLOOR) - 14 - frac;
    double v = scaled_total(t, e, os);
    double *cp = map.ml0 ? C + (m % map.ml0) * map.ms0 + (m / map.ml0) * map.ms1 +
                               (n % map.nl0) * map.ns0 + (n / map.nl0) * map.ns1
                         : C + m + n * ldc;
    if (beta != 0.0) v = fma(beta, *cp, v);
    *cp = v;
  }
}

// persistent grid: one CTA per SM (shared memory and TMEM allow no more)
unsigned emu_grid(const Context &ctx, int64_t units) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(units, std::max(ctx.sm_count, 1)));
}

struct EmuPlan {
  int mt, nt, kt, kc_blocks, ksplit, kb_per_split, frac;
};

// Tiles, exact-chunk length, K-split and fixed-point width of one GEMM.
// The int64 total of an output gathers nchunks chunk sums, each below
// ~2^(23 + frac); frac = min(29, 38 - ceil(log2 nchunks)) keeps it below 2^62.
// Small M x N with long K is split over K so that at least two CTAs per SM
// have work; the split totals are exact, so the split does not change the
// result.
EmuPlan emu_plan(int S, int64_t M, int64_t N, int64_t K, int sm_count,
                 bool allow_split, int max_split = 64) {
  EmuPlan p{};
  p.mt = (int)((M + TM - 1) / TM);
  p.nt = (int)((N + TN - 1) / TN);
  p.kt = (int)((K + KB - 1) / KB);
  p.kc_blocks = (S <= 6 ? 512 : 256) / KB;
  const int nchunks = (p.kt + p.kc_blocks - 1) / p.kc_blocks;
  int lg = 0;
  while ((1 << lg) < nchunks) ++lg;
  p.frac = std::min(FRAC, 38 - lg);
  // K-split: the persistent grid of G CTAs runs ceil(units / G) rounds of
  // cps chunks each; pick the split that minimises that, plus the cost of
  // the split-total reduction (ks int64 partials per output), so that the
  // last round of a few-tile GEMM is not mostly idle
  const int64_t ctas = (int64_t)p.mt * p.nt;
  const int64_t G = std::max(sm_count, 1);
  // one chunk of one tile: 21 * 2 * 128 * 64 * 512 bf16 flop at ~1.6 PF/s / G
  const double chunk_s = (double)S * (S + 1) * 128.0 * 64.0 * p.kc_blocks * KB /
                         (1.6e15 / (double)G);
  int best_cps = nchunks;
  double best_t = 1e300;
  const int max_ks = allow_split ? std::max(1, std::min(nchunks, std::min(max_split, 64))) : 1;
  for (int ks = 1; ks <= max_ks; ++ks) {
    const int cps = (nchunks + ks - 1) / ks;
    const int kse = (nchunks + cps - 1) / cps;
    if (kse != ks) continue;  // same split as a smaller ks
    const double rounds = (double)((ctas * kse + G - 1) / G);
    double t = rounds * cps * chunk_s;
    if (kse > 1) t += 16.0 * (double)M * (double)N * (kse + 1) / 6.0e12;  // reduce
    if (t < best_t * 0.97) {
      best_t = t;
      best_cps = cps;
    }
  }
  p.kb_per_split = best_cps * p.kc_blocks;
  p.ksplit = (p.kt + p.kb_per_split - 1) / p.kb_per_split;
  return p;
}

template <int S>
void run_emu(Context &ctx, bool ta, bool tb, int64_t M, int64_t N, int64_t K,
             double alpha, const double *A, int64_t lda, const double *B,
             int64_t ldb, double beta, double *C, int64_t ldc,
             const OutMap &map = OutMap{}) {
  const EmuPlan P = emu_plan(S, M, N, K, ctx.sm_count, true, ctx.emu_max_ksplit);
  const int mt = P.mt, nt = P.nt, kt = P.kt;
  require((int64_t)mt * nt * P.ksplit < (1LL << 31), "emu gemm: grid too large");
  // strides of op(A)(m,k) and op(B)^T(n,k)
  const int64_t ars = ta ? lda : 1, aks = ta ? 1 : lda;
  const int64_t brs = tb ? 1 : ldb, bks = tb ? ldb : 1;
  DBuf ea(ctx, sizeof(int) * M), eb(ctx, sizeof(int) * N);
  DBuf asl(ctx, (size_t)S * mt * kt * A_TILE), bsl(ctx, (size_t)S * nt * kt * B_TILE);
  DBuf wsp;
  if (P.ksplit > 1) wsp.alloc(ctx, sizeof(long long) * P.ksplit * M * N);
  int *err = ctx.device_error_word();
  auto exponents = [&](const double *p, int64_t R, int64_t rs, int64_t ks, int *e) {
    GBCC_CUDA(cudaMemsetAsync(e, 0x80, sizeof(int) * R, ctx.stream));
    if (rs == 1) {
      const int64_t kchunk = std::max<int64_t>(64, (K + 4095) / 4096);
      const dim3 grid((unsigned)((R + 127) / 128), (unsigned)((K + kchunk - 1) / kchunk));
      exponent_rows_contig_kernel<<<grid, 128, 0, ctx.stream>>>(p, R, K, ks, kchunk, e, IdxMap{});
    } else {
      const int64_t kchunk = std::max<int64_t>(1024, (K + 4095) / 4096);
      const dim3 grid((unsigned)((R + 7) / 8), (unsigned)((K + kchunk - 1) / kchunk));
      exponent_rows_warp_kernel<<<grid, 256, 0, ctx.stream>>>(p, R, K, rs, ks, kchunk, e, IdxMap{});
    }
    GBCC_CHECK_LAUNCH(ctx);
  };
  exponents(A, M, ars, aks, ea.as<int>());
  exponents(B, N, brs, bks, eb.as<int>());
  auto grid_for = [&](int64_t segs) {
    require(segs < (1LL << 31), "emulated GEMM: operand too large to split");
    int64_t g = (segs + 255) / 256;
    const int64_t cap = (int64_t)std::max(ctx.sm_count, 1) * 16;
    return (unsigned)std::max<int64_t>(1, std::min(g, cap));
  };
  split_kernel<S, TM><<<grid_for((int64_t)mt * TM * kt * 4), 256, 0, ctx.stream>>>(
      A, M, K, ars, aks, ea.as<int>(), mt, kt, asl.as<__nv_bfloat16>(), IdxMap{});
  GBCC_CHECK_LAUNCH(ctx);
  split_kernel<S, TN><<<grid_for((int64_t)nt * TN * kt * 4), 256, 0, ctx.stream>>>(
      B, N, K, brs, bks, eb.as<int>(), nt, kt, bsl.as<__nv_bfloat16>(), IdxMap{});
  GBCC_CHECK_LAUNCH(ctx);
  constexpr int STAGE_BYTES = S * (A_TILE + B_TILE);
  constexpr int STAGES = (SMEM_BUDGET / STAGE_BYTES) > 4 ? 4 : (SMEM_BUDGET / STAGE_BYTES);
  const int smem = STAGES * STAGE_BYTES;
  static bool attr_set = false;
  if (!attr_set) {
    GBCC_CUDA(cudaFuncSetAttribute(emu_gemm_kernel<S, false>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    attr_set = true;
  }
  EmuArgs args{};
  args.A = asl.as<__nv_bfloat16>();
  args.B = bsl.as<__nv_bfloat16>();
  args.ea = ea.as<int>();
  args.eb = eb.as<int>();
  args.C = C;
  args.M = M; args.N = N; args.ldc = ldc;
  args.mt = mt; args.nt = nt; args.kt = kt;
  args.kc_blocks = P.kc_blocks;
  args.kb_per_split = P.kb_per_split;
  args.ksplit = P.ksplit;
  args.frac = P.frac;
  args.W = P.ksplit > 1 ? wsp.as<long long>() : nullptr;
  if (map.ml0 > 0) {
    require(map.ml0 < (1LL << 31) && map.nl0 > 0 && map.nl0 < (1LL << 31),
            "emulated GEMM: output map needs 32-bit index lengths");
    args.mapped = 1;
    args.ml0 = (unsigned)map.ml0;
    args.nl0 = (unsigned)map.nl0;
    args.ms0 = map.ms0;
    args.ms1 = map.ms1;
    args.ns0 = map.ns0;
    args.ns1 = map.ns1;
  }
  args.os = out_scale(alpha);
  args.inject_wait = ctx.take_fault(GBCC_FAULT_DEVICE_WAIT) ? 1 : 0;
  args.beta = beta;
  args.err = err;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  if (ctx.prof) {
    ev0 = ctx.prof_event();
    ev1 = ctx.prof_event();
    GBCC_CUDA(cudaEventRecord(ev0, ctx.stream));
  }
  emu_gemm_kernel<S, false><<<emu_grid(ctx, (int64_t)mt * nt * P.ksplit), NUM_THREADS, smem,
                       ctx.stream>>>(args);
  GBCC_CHECK_LAUNCH(ctx);
  if (ctx.prof) {
    GBCC_CUDA(cudaEventRecord(ev1, ctx.stream));
    // algorithmic tensor-core work of the scheme: S(S+1)/2 bf16 products of
    // the unpadded M x N x K problem
    const double f = 2.0 * (double)M * (double)N * (double)K;
    ctx.prof_recs.push_back({ev0, ev1, f * S * (S + 1) / 2.0, f, M, N, K});
  }
  if (P.ksplit > 1) {
    const int64_t n = M * N;
    const int64_t g = std::min<int64_t>((n + 255) / 256, (int64_t)std::max(ctx.sm_count, 1) * 8);
    emu_splitk_reduce_kernel<<<(unsigned)std::max<int64_t>(g, 1), 256, 0, ctx.stream>>>(
        wsp.as<long long>(), P.ksplit, M, N, ea.as<int>(), eb.as<int>(), P.frac, args.os,
        beta, C, ldc, map);
    GBCC_CHECK_LAUNCH(ctx);
  }
  // a bounded wait that gave up sets the context's sticky error word; it is
  // read at the next synchronisation point (check_device_errors)
}

}  // namespace

// ------------------------------------------------------------ pre-split panels
// A family of `count` operands with the same shape, operand p at base +
// p*pstride, each R x K with element (r, k) at r*rs + k*ks, split once into
// digit panels (A role: 128-row tiles, B role: 64-row tiles) and reused by
// many GEMMs.
namespace {
template <int S>
void split_batch(Context &ctx, EmuPanels &P, const double *base, int64_t pstride) {
  const int TR = P.role_a ? TM : TN;
  const int64_t plane = (int64_t)P.rt * P.kt * TR * KB;  // elements per digit plane
  const int64_t K = P.K;
  auto grid_for = [&](int64_t segs) {
    require(segs < (1LL << 31), "emulated GEMM: operand too large to split");
    int64_t g = (segs + 255) / 256;
    const int64_t cap = (int64_t)std::max(ctx.sm_count, 1) * 16;
    return (unsigned)std::max<int64_t>(1, std::min(g, cap));
  };
  for (int p = 0; p < P.count; ++p) {
    const double *b = base + p * pstride;
    int *e = P.exps.as<int>() + (int64_t)p * P.rows;
    GBCC_CUDA(cudaMemsetAsync(e, 0x80, sizeof(int) * P.rows, ctx.stream));
    if (P.rs == 1) {
      const int64_t kchunk = std::max<int64_t>(64, (K + 4095) / 4096);
      const dim3 grid((unsigned)((P.rows + 127) / 128), (unsigned)((K + kchunk - 1) / kchunk));
      exponent_rows_contig_kernel<<<grid, 128, 0, ctx.stream>>>(b, P.rows, K, P.ks, kchunk, e, P.map);
    } else {
      const int64_t kchunk = std::max<int64_t>(1024, (K + 4095) / 4096);
      const dim3 grid((unsigned)((P.rows + 7) / 8), (unsigned)((K + kchunk - 1) / kchunk));
      exponent_rows_warp_kernel<<<grid, 256, 0, ctx.stream>>>(b, P.rows, K, P.rs, P.ks, kchunk, e, P.map);
    }
    GBCC_CHECK_LAUNCH(ctx);
    __nv_bfloat16 *out = P.panels.as<__nv_bfloat16>() + (int64_t)p * S * plane;
    if (P.role_a)
      split_kernel<S, TM><<<grid_for((int64_t)P.rt * TM * P.kt * 4), 256, 0, ctx.stream>>>(
          b, P.rows, K, P.rs, P.ks, e, P.rt, P.kt, out, P.map);
    else
      split_kernel<S, TN><<<grid_for((int64_t)P.rt * TN * P.kt * 4), 256, 0, ctx.stream>>>(
          b, P.rows, K, P.rs, P.ks, e, P.rt, P.kt, out, P.map);
    GBCC_CHECK_LAUNCH(ctx);
  }
}

template <int S>
void gemm_panels(Context &ctx, const EmuPanels &A, int ia, const EmuPanels &B, int ib,
                 double alpha, double beta, double *C, df32 *Cdf, int64_t ldc,
                 const OutMap &map = OutMap{}) {
  const int64_t M = A.rows, N = B.rows, K = A.K;
  // float-float output is written directly (no K-split workspace)
  const EmuPlan P = emu_plan(S, M, N, K, ctx.sm_count, Cdf == nullptr, ctx.emu_max_ksplit);
  const int64_t aplane = (int64_t)A.rt * A.kt * TM * KB;
  const int64_t bplane = (int64_t)B.rt * B.kt * TN * KB;
  DBuf wsp;
  if (P.ksplit > 1) wsp.alloc(ctx, sizeof(long long) * P.ksplit * M * N);
  constexpr int STAGE_BYTES = S * (A_TILE + B_TILE);
  constexpr int STAGES = (SMEM_BUDGET / STAGE_BYTES) > 4 ? 4 : (SMEM_BUDGET / STAGE_BYTES);
  const int smem = STAGES * STAGE_BYTES;
  void (*kern)(EmuArgs) = Cdf ? emu_gemm_kernel<S, true> : emu_gemm_kernel<S, false>;
  GBCC_CUDA(cudaFuncSetAttribute(kern,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  EmuArgs args{};
  args.A = A.panels.as<__nv_bfloat16>() + (int64_t)ia * S * aplane;
  args.B = B.panels.as<__nv_bfloat16>() + (int64_t)ib * S * bplane;
  args.ea = A.exps.as<int>() + (int64_t)ia * M;
  args.eb = B.exps.as<int>() + (int64_t)ib * N;
  args.C = C;
  args.Cdf = Cdf;
  args.M = M; args.N = N; args.ldc = ldc;
  args.mt = P.mt; args.nt = P.nt; args.kt = P.kt;
  args.kc_blocks = P.kc_blocks;
  args.kb_per_split = P.kb_per_split;
  args.ksplit = P.ksplit;
  args.frac = P.frac;
  args.W = P.ksplit > 1 ? wsp.as<long long>() : nullptr;
  if (map.ml0 > 0) {
    require(Cdf == nullptr && map.ml0 < (1LL << 31) && map.nl0 > 0 && map.nl0 < (1LL << 31),
            "emulated GEMM: output map needs FP64 output and 32-bit index lengths");
    args.mapped = 1;
    args.ml0 = (unsigned)map.ml0;
    args.nl0 = (unsigned)map.nl0;
    args.ms0 = map.ms0;
    args.ms1 = map.ms1;
    args.ns0 = map.ns0;
    args.ns1 = map.ns1;
  }
  args.os = out_scale(alpha);
  args.inject_wait = ctx.take_fault(GBCC_FAULT_DEVICE_WAIT) ? 1 : 0;
  args.beta = beta;
  args.err = ctx.device_error_word();
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  if (ctx.prof) {
    ev0 = ctx.prof_event();
    ev1 = ctx.prof_event();
    GBCC_CUDA(cudaEventRecord(ev0, ctx.stream));
  }
  kern<<<emu_grid(ctx, (int64_t)P.mt * P.nt * P.ksplit), NUM_THREADS, smem,
                       ctx.stream>>>(args);
  GBCC_CHECK_LAUNCH(ctx);
  if (ctx.prof) {
    GBCC_CUDA(cudaEventRecord(ev1, ctx.stream));
    const double f = 2.0 * (double)M * (double)N * (double)K;
    ctx.prof_recs.push_back({ev0, ev1, f * S * (S + 1) / 2.0, f, M, N, K});
  }
  if (P.ksplit > 1) {
    const int64_t n = M * N;
    const int64_t g = std::min<int64_t>((n + 255) / 256, (int64_t)std::max(ctx.sm_count, 1) * 8);
    emu_splitk_reduce_kernel<<<(unsigned)std::max<int64_t>(g, 1), 256, 0, ctx.stream>>>(
        wsp.as<long long>(), P.ksplit, M, N, args.ea, args.eb, P.frac, args.os, beta, C, ldc, map);
    GBCC_CHECK_LAUNCH(ctx);
  }
  ctx.flops += 2.0 * (double)M * (double)N * (double)K;
}
// Grouped launch over panels: problem q multiplies operand ia[q] of A with
// operand ib[q] of B into C[q] (Cdf[q] for float-float output); all problems
// share M, N, K, alpha, beta and ldc.  One persistent launch walks the tiles
// of every problem, so a batch of small or short-K products fills the GPU
// and pays one launch.
// Without ia and ib (strided batch) problem q multiplies operand q of A with
// operand q of B into C[0] + q sC: no table is uploaded, so the launch can be
// captured into a graph.
template <int S>
void gemm_panels_grouped(Context &ctx, const EmuPanels &A, const int *ia, const EmuPanels &B,
                         const int *ib, int nprob, double alpha, double beta,
                         double *const *C, df32 *const *Cdf, int64_t ldc, int64_t sC = 0,
                         const OutMap &map = OutMap{}) {
  const int64_t M = A.rows, N = B.rows, K = A.K;
  const EmuPlan P = emu_plan(S, M, N, K, ctx.sm_count, false);
  require((int64_t)P.mt * P.nt * nprob < (1LL << 31), "grouped GEMM: too many tiles");
  const int64_t aplane = (int64_t)A.rt * A.kt * TM * KB;
  const int64_t bplane = (int64_t)B.rt * B.kt * TN * KB;
  const bool strided = ia == nullptr;
  DBuf table;
  if (!strided) {
    std::vector<EmuProb> probs((size_t)nprob);
    for (int q = 0; q < nprob; ++q) {
      require(ia[q] >= 0 && ia[q] < A.count && ib[q] >= 0 && ib[q] < B.count,
              "grouped GEMM: operand index");
      EmuProb &e = probs[q];
      e.A = A.panels.as<__nv_bfloat16>() + (int64_t)ia[q] * S * aplane;
      e.B = B.panels.as<__nv_bfloat16>() + (int64_t)ib[q] * S * bplane;
      e.ea = A.exps.as<int>() + (int64_t)ia[q] * M;
      e.eb = B.exps.as<int>() + (int64_t)ib[q] * N;
      e.C = C ? C[q] : nullptr;
      e.Cdf = Cdf ? Cdf[q] : nullptr;
    }
    // a copy from pageable memory has read its source when it returns, but
    // a captured one would read it again at every replay
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    GBCC_CUDA(cudaStreamIsCapturing(ctx.stream, &cap));
    require(cap == cudaStreamCaptureStatusNone,
            "grouped GEMM: a problem table cannot be captured into a graph");
    table.alloc(ctx, sizeof(EmuProb) * probs.size());
    GBCC_CUDA(cudaMemcpyAsync(table.as<EmuProb>(), probs.data(),
                              sizeof(EmuProb) * probs.size(), cudaMemcpyHostToDevice,
                              ctx.stream));
  } else {
    require(nprob <= A.count && nprob <= B.count, "batched GEMM: operand count");
  }
  constexpr int STAGE_BYTES = S * (A_TILE + B_TILE);
  constexpr int STAGES = (SMEM_BUDGET / STAGE_BYTES) > 4 ? 4 : (SMEM_BUDGET / STAGE_BYTES);
  const int smem = STAGES * STAGE_BYTES;
  void (*kern)(EmuArgs) = Cdf ? emu_gemm_kernel<S, true> : emu_gemm_kernel<S, false>;
  GBCC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  EmuArgs args{};
  args.M = M; args.N = N; args.ldc = ldc;
  args.mt = P.mt; args.nt = P.nt; args.kt = P.kt;
  args.kc_blocks = P.kc_blocks;
  args.kb_per_split = P.kb_per_split;
  args.ksplit = 1;
  args.frac = P.frac;
  args.os = out_scale(alpha);
  args.inject_wait = ctx.take_fault(GBCC_FAULT_DEVICE_WAIT) ? 1 : 0;
  args.beta = beta;
  args.err = ctx.device_error_word();
  args.nprob = nprob;
  if (strided) {
    args.A = A.panels.as<__nv_bfloat16>();
    args.B = B.panels.as<__nv_bfloat16>();
    args.ea = A.exps.as<int>();
    args.eb = B.exps.as<int>();
    args.C = C ? C[0] : nullptr;
    args.Cdf = Cdf ? Cdf[0] : nullptr;
    args.qsA = S * aplane;
    args.qsB = S * bplane;
    args.qsea = M;
    args.qseb = N;
    args.qsC = sC;
    if (map.ml0 > 0) {
      require(Cdf == nullptr && map.ml0 < (1LL << 31) && map.nl0 > 0 &&
                  map.nl0 < (1LL << 31),
              "batched GEMM: output map needs FP64 output and 32-bit index lengths");
      args.mapped = 1;
      args.ml0 = (unsigned)map.ml0;
      args.nl0 = (unsigned)map.nl0;
      args.ms0 = map.ms0;
      args.ms1 = map.ms1;
      args.ns0 = map.ns0;
      args.ns1 = map.ns1;
    }
  } else {
    require(map.ml0 == 0, "grouped GEMM: no output map with a problem table");
    args.probs = table.as<EmuProb>();
  }
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  if (ctx.prof) {
    ev0 = ctx.prof_event();
    ev1 = ctx.prof_event();
    GBCC_CUDA(cudaEventRecord(ev0, ctx.stream));
  }
  kern<<<emu_grid(ctx, (int64_t)P.mt * P.nt * nprob), NUM_THREADS, smem, ctx.stream>>>(args);
  GBCC_CHECK_LAUNCH(ctx);
  const double f = 2.0 * (double)M * (double)N * (double)K * nprob;
  if (ctx.prof) {
    GBCC_CUDA(cudaEventRecord(ev1, ctx.stream));
    ctx.prof_recs.push_back({ev0, ev1, f * S * (S + 1) / 2.0, f, M, N, K * nprob});
  }
  ctx.flops += f;
}
}  // namespace

void emu_gemm_panels_batched(Context &ctx, const EmuPanels &A, const EmuPanels &B, int nprob,
                             double alpha, double beta, double *C, int64_t ldc, int64_t sC,
                             const OutMap &map) {
  require(nprob >= 1, "batched GEMM: no problems");
  require(A.role_a && !B.role_a && A.K == B.K && A.S == B.S, "batched GEMM: operand mismatch");
  // a few-tile product with long K keeps its K-split, problem by problem,
  // unless the batch alone fills the GPU with tiles
  const EmuPlan P1 = emu_plan(A.S, A.rows, B.rows, A.K, ctx.sm_count, true, ctx.emu_max_ksplit);
  if (P1.ksplit > 1 && (int64_t)P1.mt * P1.nt * nprob < ctx.sm_count) {
    for (int q = 0; q < nprob; ++q) {
      if (map.ml0 > 0)
        emu_gemm_panels_mapped(ctx, A, q, B, q, alpha, beta, C + (int64_t)q * sC, map);
      else
        emu_gemm_panels(ctx, A, q, B, q, alpha, beta, C + (int64_t)q * sC, ldc);
    }
    return;
  }
  double *const Cs[1] = {C};
  switch (A.S) {
    case 4: gemm_panels_grouped<4>(ctx, A, nullptr, B, nullptr, nprob, alpha, beta, Cs, nullptr, ldc, sC, map); break;
    case 5: gemm_panels_grouped<5>(ctx, A, nullptr, B, nullptr, nprob, alpha, beta, Cs, nullptr, ldc, sC, map); break;
    case 6: gemm_panels_grouped<6>(ctx, A, nullptr, B, nullptr, nprob, alpha, beta, Cs, nullptr, ldc, sC, map); break;
    case 7: gemm_panels_grouped<7>(ctx, A, nullptr, B, nullptr, nprob, alpha, beta, Cs, nullptr, ldc, sC, map); break;
    case 8: gemm_panels_grouped<8>(ctx, A, nullptr, B, nullptr, nprob, alpha, beta, Cs, nullptr, ldc, sC, map); break;
    default: throw Error(GBCC_BAD_ARG, "emu_slices must be in [4, 8]");
  }
}

void emu_gemm_panels_grouped(Context &ctx, const EmuPanels &A, const int *ia,
                             const EmuPanels &B, const int *ib, int nprob, double alpha,
                             double beta, double *const *C, df32 *const *Cdf, int64_t ldc) {
  require(nprob >= 1, "grouped GEMM: no problems");
  require(ia != nullptr && ib != nullptr, "grouped GEMM: operand indices");
  require(A.role_a && !B.role_a && A.K == B.K && A.S == B.S, "grouped GEMM: operand mismatch");
  require((C == nullptr) != (Cdf == nullptr), "grouped GEMM: one output kind");
  if (Cdf)
    require(out_scale(alpha).pow2 && (beta == 0.0 || beta == 1.0),
            "grouped GEMM: float-float output needs alpha = +-2^k and beta in {0, 1}");
  switch (A.S) {
    case 4: gemm_panels_grouped<4>(ctx, A, ia, B, ib, nprob, alpha, beta, C, Cdf, ldc); break;
    case 5: gemm_panels_grouped<5>(ctx, A, ia, B, ib, nprob, alpha, beta, C, Cdf, ldc); break;
    case 6: gemm_panels_grouped<6>(ctx, A, ia, B, ib, nprob, alpha, beta, C, Cdf, ldc); break;
    case 7: gemm_panels_grouped<7>(ctx, A, ia, B, ib, nprob, alpha, beta, C, Cdf, ldc); break;
    case 8: gemm_panels_grouped<8>(ctx, A, ia, B, ib, nprob, alpha, beta, C, Cdf, ldc); break;
    default: throw Error(GBCC_BAD_ARG, "emu_slices must be in [4, 8]");
  }
}

EmuPanels emu_panels_alloc(Context &ctx, bool role_a, int64_t R, int64_t K) {
  require(R > 0 && K > 0, "emu_panels_alloc: empty operand");
  EmuPanels P;
  P.role_a = role_a;
  P.S = ctx.emu_slices;
  P.rows = R;
  P.K = K;
  P.count = 1;
  P.rt = (int)((R + (role_a ? TM : TN) - 1) / (role_a ? TM : TN));
  P.kt = (int)((K + KB - 1) / KB);
  P.panels.alloc(ctx, (size_t)P.S * P.rt * P.kt * (role_a ? A_TILE : B_TILE));
  P.exps.alloc(ctx, sizeof(int) * (size_t)R);
  return P;
}

void ladder_amax(Context &ctx, const double *dG, int64_t G, int64_t Nv, void *amax) {
  GBCC_CUDA(cudaMemsetAsync(amax, 0, sizeof(unsigned long long) * Nv, ctx.stream));
  const int64_t ncol = Nv * Nv;
  column_norm_max_kernel<<<(unsigned)((ncol * 32 + 255) / 256), 256, 0, ctx.stream>>>(
      dG, G, ncol, Nv, static_cast<unsigned long long *>(amax));
  GBCC_CHECK_LAUNCH(ctx);
}

void ladder_row_exponents(Context &ctx, const void *amax, int64_t x0, int64_t nx, int64_t y0,
                          int64_t ny, int *er) {
  const int64_t R = nx * ny;
  ladder_row_exponent_kernel<<<(unsigned)((R + 255) / 256), 256, 0, ctx.stream>>>(
      static_cast<const unsigned long long *>(amax), x0, nx, y0, ny, er);
  GBCC_CHECK_LAUNCH(ctx);
}

namespace {
// The panel-output launch from operand panels (A rows M = A.rows, B rows
// N = B.rows, K): V = A B^T written as the digits of P (see EmuArgs).
template <int S>
void launch_to_panels(Context &ctx, const __nv_bfloat16 *Ap, const int *ea,
                      const __nv_bfloat16 *Bp, const int *eb, int64_t M, int64_t N, int64_t K,
                      unsigned px, unsigned pd, EmuPanels &P) {
  const EmuPlan pl = emu_plan(S, M, N, K, ctx.sm_count, false);
  const int mt = pl.mt, nt = pl.nt, kt = pl.kt;
  require((int64_t)mt * nt < (1LL << 31), "emu gemm: grid too large");
  // rows past R are never written: give them the digits of zero
  if (P.rows % TM != 0) {
    const int64_t pad = (int64_t)P.rt * TM - P.rows;
    const int64_t n = pad * P.kt * (KB / 8) * S;
    const unsigned g = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>((n + 255) / 256, (int64_t)std::max(ctx.sm_count, 1) * 16));
    zero_panel_rows_kernel<<<g, 256, 0, ctx.stream>>>(P.panels.as<__nv_bfloat16>(), P.rows,
                                                      P.rt, P.kt, S,
                                                      (int64_t)P.rt * P.kt * TM * KB);
    GBCC_CHECK_LAUNCH(ctx);
  }
  constexpr int STAGE_BYTES = S * (A_TILE + B_TILE);
  constexpr int STAGES = (SMEM_BUDGET / STAGE_BYTES) > 4 ? 4 : (SMEM_BUDGET / STAGE_BYTES);
  const int smem = STAGES * STAGE_BYTES;
  GBCC_CUDA(cudaFuncSetAttribute(emu_gemm_kernel<S, false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  EmuArgs args{};
  args.A = Ap;
  args.B = Bp;
  args.ea = ea;
  args.eb = eb;
  args.M = M; args.N = N; args.ldc = 0;
  args.mt = mt; args.nt = nt; args.kt = kt;
  args.kc_blocks = pl.kc_blocks;
  args.kb_per_split = pl.kb_per_split;
  args.ksplit = 1;
  args.frac = pl.frac;
  args.os = out_scale(1.0);
  args.inject_wait = ctx.take_fault(GBCC_FAULT_DEVICE_WAIT) ? 1 : 0;
  args.beta = 0.0;
  args.err = ctx.device_error_word();
  args.pout = P.panels.as<__nv_bfloat16>();
  args.pexp = P.exps.as<int>();
  args.prt = P.rt;
  args.pkt = P.kt;
  args.px = px;
  args.pd = pd;
  args.pplane = (int64_t)P.rt * P.kt * TM * KB;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  if (ctx.prof) {
    ev0 = ctx.prof_event();
    ev1 = ctx.prof_event();
    GBCC_CUDA(cudaEventRecord(ev0, ctx.stream));
  }
  emu_gemm_kernel<S, false><<<emu_grid(ctx, (int64_t)mt * nt), NUM_THREADS, smem,
                              ctx.stream>>>(args);
  GBCC_CHECK_LAUNCH(ctx);
  if (ctx.prof) {
    GBCC_CUDA(cudaEventRecord(ev1, ctx.stream));
    const double f = 2.0 * (double)M * (double)N * (double)K;
    ctx.prof_recs.push_back({ev0, ev1, f * S * (S + 1) / 2.0, f, M, N, K});
  }
}

}  // namespace

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
  require(M < (1LL << 31) && N < (1LL << 31), "emu_gemm_panels_to_panels: size");
  const int64_t aplane = (int64_t)A.rt * A.kt * TM * KB;
  const int64_t bplane = (int64_t)B.rt * B.kt * TN * KB;
  const __nv_bfloat16 *Ap = A.panels.as<__nv_bfloat16>() + (int64_t)ia * A.S * aplane;
  const __nv_bfloat16 *Bp = B.panels.as<__nv_bfloat16>() + (int64_t)ib * B.S * bplane;
  const int *ea = A.exps.as<int>() + (int64_t)ia * M;
  const int *eb = B.exps.as<int>() + (int64_t)ib * N;
  switch (A.S) {
    case 4: launch_to_panels<4>(ctx, Ap, ea, Bp, eb, M, N, K, (unsigned)px, (unsigned)pd, P); break;
    case 5: launch_to_panels<5>(ctx, Ap, ea, Bp, eb, M, N, K, (unsigned)px, (unsigned)pd, P); break;
    case 6: launch_to_panels<6>(ctx, Ap, ea, Bp, eb, M, N, K, (unsigned)px, (unsigned)pd, P); break;
    case 7: launch_to_panels<7>(ctx, Ap, ea, Bp, eb, M, N, K, (unsigned)px, (unsigned)pd, P); break;
    case 8: launch_to_panels<8>(ctx, Ap, ea, Bp, eb, M, N, K, (unsigned)px, (unsigned)pd, P); break;
    default: throw Error(GBCC_BAD_ARG, "emu_slices must be in [4, 8]");
  }
  ctx.flops += 2.0 * (double)M * (double)N * (double)K;
}

EmuPanels emu_split(Context &ctx, bool role_a, const double *base, int64_t R,
                    int64_t K, int64_t rs, int64_t ks, int count, int64_t pstride,
                    const IdxMap &map) {
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
  P.rt = (int)((R + (role_a ? TM : TN) - 1) / (role_a ? TM : TN));
  P.kt = (int)((K + KB - 1) / KB);
  const size_t tile = role_a ? A_TILE : B_TILE;
  P.panels.alloc(ctx, (size_t)count * P.S * P.rt * P.kt * tile);
  P.exps.alloc(ctx, sizeof(int) * (size_t)count * R);
  switch (P.S) {
    case 4: split_batch<4>(ctx, P, base, pstride); break;
    case 5: split_batch<5>(ctx, P, base, pstride); break;
    case 6: split_batch<6>(ctx, P, base, pstride); break;
    case 7: split_batch<7>(ctx, P, base, pstride); break;
    case 8: split_batch<8>(ctx, P, base, pstride); break;
    default: throw Error(GBCC_BAD_ARG, "emu_slices must be in [4, 8]");
  }
  return P;
}

void emu_gemm_panels_mapped(Context &ctx, const EmuPanels &A, int ia, const EmuPanels &B,
                            int ib, double alpha, double beta, double *C, const OutMap &map) {
  require(A.role_a && !B.role_a && A.K == B.K && A.S == B.S,
          "emu_gemm_panels_mapped: operand mismatch");
  require(ia >= 0 && ia < A.count && ib >= 0 && ib < B.count, "emu_gemm_panels_mapped: index");
  require(map.ml0 > 0 && map.nl0 > 0, "emu_gemm_panels_mapped: empty map");
  switch (A.S) {
    case 4: gemm_panels<4>(ctx, A, ia, B, ib, alpha, beta, C, nullptr, 0, map); break;
    case 5: gemm_panels<5>(ctx, A, ia, B, ib, alpha, beta, C, nullptr, 0, map); break;
    case 6: gemm_panels<6>(ctx, A, ia, B, ib, alpha, beta, C, nullptr, 0, map); break;
    case 7: gemm_panels<7>(ctx, A, ia, B, ib, alpha, beta, C, nullptr, 0, map); break;
    case 8: gemm_panels<8>(ctx, A, ia, B, ib, alpha, beta, C, nullptr, 0, map); break;
    default: throw Error(GBCC_BAD_ARG, "emu_slices must be in [4, 8]");
  }
}

void emu_gemm_panels(Context &ctx, const EmuPanels &A, int ia, const EmuPanels &B,
                     int ib, double alpha, double beta, double *C, int64_t ldc,
                     df32 *Cdf) {
  require(A.role_a && !B.role_a && A.K == B.K && A.S == B.S, "emu_gemm_panels: operand mismatch");
  require(ia >= 0 && ia < A.count && ib >= 0 && ib < B.count, "emu_gemm_panels: index");
  if (Cdf) {
    require(out_scale(alpha).pow2 && (beta == 0.0 || beta == 1.0),
            "emu_gemm_panels: float-float output needs alpha = +-2^k and beta in {0, 1}");
  }
  switch (A.S) {
    case 4: gemm_panels<4>(ctx, A, ia, B, ib, alpha, beta, C, Cdf, ldc); break;
    case 5: gemm_panels<5>(ctx, A, ia, B, ib, alpha, beta, C, Cdf, ldc); break;
    case 6: gemm_panels<6>(ctx, A, ia, B, ib, alpha, beta, C, Cdf, ldc); break;
    case 7: gemm_panels<7>(ctx, A, ia, B, ib, alpha, beta, C, Cdf, ldc); break;
    case 8: gemm_panels<8>(ctx, A, ia, B, ib, alpha, beta, C, Cdf, ldc); break;
    default: throw Error(GBCC_BAD_ARG, "emu_slices must be in [4, 8]");
  }
}

void gemm_emu_mapped(Context &ctx, bool ta, bool tb, int64_t M, int64_t N, int64_t K,
                     double alpha, const double *A, int64_t lda, const double *B,
                     int64_t ldb, double *C, const OutMap &map) {
  require(map.ml0 > 0 && map.nl0 > 0, "gemm_emu_mapped: empty map");
  switch (ctx.emu_slices) {
    case 4: run_emu<4>(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, 0.0, C, 0, map); break;
    case 5: run_emu<5>(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, 0.0, C, 0, map); break;
    case 6: run_emu<6>(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, 0.0, C, 0, map); break;
    case 7: run_emu<7>(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, 0.0, C, 0, map); break;
    case 8: run_emu<8>(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, 0.0, C, 0, map); break;
    default: throw Error(GBCC_BAD_ARG, "emu_slices must be in [4, 8]");
  }
  ctx.flops += 2.0 * (double)M * (double)N * (double)K;
}

void gemm_emu(Context &ctx, bool ta, bool tb, int64_t M, int64_t N, int64_t K,
              double alpha, const double *A, int64_t lda, const double *B,
              int64_t ldb, double beta, double *C, int64_t ldc, int64_t batch,
              int64_t sA, int64_t sB, int64_t sC) {
  if (batch > 1 && batch < (1 << 20)) {
    // a batch of same-shape products: the operands of all entries are split
    // into one panel family each, and one grouped launch walks the tiles of
    // every entry
    const int64_t ars = ta ? lda : 1, aks = ta ? 1 : lda;
    const int64_t brs = tb ? 1 : ldb, bks = tb ? ldb : 1;
    EmuPanels PA = emu_split(ctx, true, A, M, K, ars, aks, (int)batch, sA);
    EmuPanels PB = emu_split(ctx, false, B, N, K, brs, bks, (int)batch, sB);
    emu_gemm_panels_batched(ctx, PA, PB, (int)batch, alpha, beta, C, ldc, sC);
    return;
  }
  for (int64_t z = 0; z < batch; ++z) {
    const double *Az = A + z * sA;
    const double *Bz = B + z * sB;
    double *Cz = C + z * sC;
    switch (ctx.emu_slices) {
      case 4: run_emu<4>(ctx, ta, tb, M, N, K, alpha, Az, lda, Bz, ldb, beta, Cz, ldc); break;
      case 5: run_emu<5>(ctx, ta, tb, M, N, K, alpha, Az, lda, Bz, ldb, beta, Cz, ldc); break;
      case 6: run_emu<6>(ctx, ta, tb, M, N, K, alpha, Az, lda, Bz, ldb, beta, Cz, ldc); break;
      case 7: run_emu<7>(ctx, ta, tb, M, N, K, alpha, Az, lda, Bz, ldb, beta, Cz, ldc); break;
      case 8: run_emu<8>(ctx, ta, tb, M, N, K, alpha, Az, lda, Bz, ldb, beta, Cz, ldc); break;
      default: throw Error(GBCC_BAD_ARG, "emu_slices must be in [4, 8]");
    }
    ctx.flops += 2.0 * (double)M * (double)N * (double)K;
  }
}

}  // namespace gbcc

// ------------------------------------------------------------------------
// Emulated GEMM that allocates nothing.
//
// Some callers of this library cannot let it allocate device memory: a
// serving process that has reserved the whole HBM budget for its own arena,
// or a host runtime whose hot loop must not enter the CUDA allocator (its
// latency and fragmentation are outside the caller's control).  For them the
// emulated GEMM can run with its scratch (row/column exponents, the digit
// panels of both operands and the error word) in one file-scope device array
// of fixed size instead of stream-ordered allocations.
//
// Limits and sharing: the array holds NOALLOC_SCRATCH_BYTES (32 MiB); every
// GPU that runs the library's kernels holds it until the process exits (with
// lazy module loading, from the first use on that GPU).  Every call on a
// device uses the same array and it keeps the previous call's contents; the
// error word is cleared at the start of each call and all other scratch is
// fully rewritten before it is read.  Calls whose work overlaps on the GPU
// (two streams, or two host threads) race on the array and must be ordered
// by the caller.  Each call reads the kernel's error word back, so it returns
// only when its GEMM has finished.  The device address of the array is looked
// up once per device, on the first call made with that device current, and
// kept for the life of the process: a device reset (cudaDeviceReset) makes
// the kept address stale, so the entry point is not for use after one.
namespace gbcc {
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = 32u << 20;
__device__ __align__(256) uint8_t g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
uint8_t *g_noalloc_ptr[MAX_DEVICES] = {};

uint8_t *noalloc_scratch(int device) {
  require(device >= 0 && device < MAX_DEVICES, "device index out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void *p = nullptr;
    // host code must not take the array's address directly: the name is a
    // host-side stand-in; the device address comes from the runtime
    GBCC_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_ptr[device] = static_cast<uint8_t *>(p);
  }
  return g_noalloc_ptr[device];
}

size_t round256(size_t x) { return (x + 255) / 256 * 256; }

template <int S>
void run_emu_static(Context &ctx, bool ta, bool tb, int64_t M, int64_t N,
                    int64_t K, double alpha, const double *A, int64_t lda,
                    const double *B, int64_t ldb, double beta, double *C,
                    int64_t ldc, uint8_t *scratch) {
  const int mt = (int)((M + TM - 1) / TM);
  const int nt = (int)((N + TN - 1) / TN);
  const int kt = (int)((K + KB - 1) / KB);
  require(nt <= 65535, "emu gemm: grid too large");
  const size_t off_ea = 256;
  const size_t off_eb = off_ea + round256(sizeof(int) * M);
  const size_t off_a = off_eb + round256(sizeof(int) * N);
  const size_t off_b = off_a + round256((size_t)S * mt * kt * A_TILE);
  const size_t need = off_b + round256((size_t)S * nt * kt * B_TILE);
  if (need > NOALLOC_SCRATCH_BYTES)
    throw Error(GBCC_BAD_ARG,
                "gbcc_dgemm_emu_noalloc: this GEMM needs " + std::to_string(need) +
                    " bytes of scratch, more than the fixed " +
                    std::to_string(NOALLOC_SCRATCH_BYTES) + " bytes");
  int *err = reinterpret_cast<int *>(scratch);
  int *ea = reinterpret_cast<int *>(scratch + off_ea);
  int *eb = reinterpret_cast<int *>(scratch + off_eb);
  __nv_bfloat16 *asl = reinterpret_cast<__nv_bfloat16 *>(scratch + off_a);
  __nv_bfloat16 *bsl = reinterpret_cast<__nv_bfloat16 *>(scratch + off_b);
  const int64_t ars = ta ? lda : 1, aks = ta ? 1 : lda;
  const int64_t brs = tb ? 1 : ldb, bks = tb ? ldb : 1;
  GBCC_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx.stream));
  auto exponents = [&](const double *p, int64_t R, int64_t rs, int64_t ks, int *e) {
    GBCC_CUDA(cudaMemsetAsync(e, 0x80, sizeof(int) * R, ctx.stream));
    if (rs == 1) {
      const int64_t kchunk = std::max<int64_t>(64, (K + 4095) / 4096);
      const dim3 grid((unsigned)((R + 127) / 128), (unsigned)((K + kchunk - 1) / kchunk));
      exponent_rows_contig_kernel<<<grid, 128, 0, ctx.stream>>>(p, R, K, ks, kchunk, e, IdxMap{});
    } else {
      const int64_t kchunk = std::max<int64_t>(1024, (K + 4095) / 4096);
      const dim3 grid((unsigned)((R + 7) / 8), (unsigned)((K + kchunk - 1) / kchunk));
      exponent_rows_warp_kernel<<<grid, 256, 0, ctx.stream>>>(p, R, K, rs, ks, kchunk, e, IdxMap{});
    }
    GBCC_CHECK_LAUNCH(ctx);
  };
  exponents(A, M, ars, aks, ea);
  exponents(B, N, brs, bks, eb);
  auto grid_for = [&](int64_t segs) {
    require(segs < (1LL << 31), "emulated GEMM: operand too large to split");
    int64_t g = (segs + 255) / 256;
    const int64_t cap = (int64_t)std::max(ctx.sm_count, 1) * 16;
    return (unsigned)std::max<int64_t>(1, std::min(g, cap));
  };
  split_kernel<S, TM><<<grid_for((int64_t)mt * TM * kt * 4), 256, 0, ctx.stream>>>(
      A, M, K, ars, aks, ea, mt, kt, asl, IdxMap{});
  GBCC_CHECK_LAUNCH(ctx);
  split_kernel<S, TN><<<grid_for((int64_t)nt * TN * kt * 4), 256, 0, ctx.stream>>>(
      B, N, K, brs, bks, eb, nt, kt, bsl, IdxMap{});
  GBCC_CHECK_LAUNCH(ctx);
  constexpr int STAGE_BYTES = S * (A_TILE + B_TILE);
  constexpr int STAGES = (SMEM_BUDGET / STAGE_BYTES) > 4 ? 4 : (SMEM_BUDGET / STAGE_BYTES);
  const int smem = STAGES * STAGE_BYTES;
  GBCC_CUDA(cudaFuncSetAttribute(emu_gemm_kernel<S, false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  EmuArgs args{};
  args.A = asl;
  args.B = bsl;
  args.ea = ea;
  args.eb = eb;
  args.C = C;
  args.M = M; args.N = N; args.ldc = ldc;
  args.mt = mt; args.nt = nt; args.kt = kt;
  {
    const EmuPlan P = emu_plan(S, M, N, K, ctx.sm_count, false);  // no K-split workspace
    args.kc_blocks = P.kc_blocks;
    args.kb_per_split = P.kb_per_split;
    args.ksplit = 1;
    args.frac = P.frac;
    args.W = nullptr;
  }
  args.os = out_scale(alpha);
  args.inject_wait = ctx.take_fault(GBCC_FAULT_DEVICE_WAIT) ? 1 : 0;
  args.beta = beta;
  args.err = err;
  emu_gemm_kernel<S, false><<<emu_grid(ctx, (int64_t)mt * nt), NUM_THREADS, smem, ctx.stream>>>(args);
  GBCC_CHECK_LAUNCH(ctx);
  int h = 0;
  GBCC_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
  GBCC_CUDA(cudaStreamSynchronize(ctx.stream));
  if (h != ERR_NONE)
    throw Error(GBCC_TIMEOUT, "emulated GEMM: a bounded device wait gave up (code " +
                                  std::to_string(h) + ")");
}

}  // namespace

void gemm_emu_noalloc(Context &ctx, bool ta, bool tb, int64_t M, int64_t N,
                      int64_t K, double alpha, const double *A, int64_t lda,
                      const double *B, int64_t ldb, double beta, double *C,
                      int64_t ldc) {
  require(M > 0 && N > 0 && K > 0, "gbcc_dgemm_emu_noalloc: sizes must be positive");
  require(A && B && C, "gbcc_dgemm_emu_noalloc: null operand");
  uint8_t *scratch = noalloc_scratch(ctx.device);
  switch (ctx.emu_slices) {
    case 4: run_emu_static<4>(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, scratch); break;
    case 5: run_emu_static<5>(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, scratch); break;
    case 6: run_emu_static<6>(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, scratch); break;
    case 7: run_emu_static<7>(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, scratch); break;
    case 8: run_emu_static<8>(ctx, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, scratch); break;
    default: throw Error(GBCC_BAD_ARG, "emu_slices must be in [4, 8]");
  }
  ctx.flops += 2.0 * (double)M * (double)N * (double)K;
}

}  // namespace gbcc
