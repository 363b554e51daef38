// hqr_ozaki.cuh -- split-precision trailing updates on the 5th-generation
// tensor cores (tcgen05, TMEM accumulators, bulk-TMA operand staging).
//
// A block reflector is applied as three products (D = C_top + V^T C_bot,
// D2 = T^T D, C -= [I|V] D2 -- the CORE_dtsmqr / CORE_dormqr arithmetic with
// the full NB x NB T), each computed as an Ozaki-style sum of exact slice
// products (Ozaki, Ogita, Oishi, Rump, "Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59, 2012):
//
//   * every row of the left operand X (and every column of the right
//     operand Y) is scaled by the power of two of its largest element and
//     written as a fixed-point integer F with |F| < 2^55;
//   * F is split into kSlices signed digits of kRho = 7 bits, |d| <= 64,
//     F = sum_p d_p 2^(56 - 7p); every digit is an exact BF16 value;
//   * the slice products X_p Y_q with p + q <= kSlices + 1 are exact on the
//     tensor cores: |d_x d_y| <= 2^12, a K = NB <= 256 sum stays below 2^20,
//     and the <= 8 products sharing t = p + q (same weight 2^(-7t)) are
//     accumulated in one FP32 TMEM accumulator, < 2^23 < 2^24;
//   * the 8 t-group accumulators (8 x 64 TMEM columns = the whole TMEM) are
//     recombined exactly in 64-bit integers (two Horner chains in base 2^7),
//     converted to FP64 once and scaled back: 2 FP64 operations per output.
//
// The left operands (V^T, T^T, V of a panel tile) are sliced once per panel
// tile into HBM, already in the tcgen05 K-major core-matrix layout, so an
// update streams each 16-deep K chunk of all 8 slices with one 32 KiB bulk
// TMA copy.  The right operand (a 64-column block of the trailing tile) is
// sliced on the fly by the CTA into shared memory.  MMAs are issued by one
// thread (M = 128, N = 64, K = 16, BF16 x BF16 -> FP32) into the 8
// accumulators; the K loop is double-buffered (TMA + slicing of chunk k+1
// overlap the MMAs of chunk k).  Every mbarrier wait is bounded; on time-out
// the kernel's error word is set and the task is abandoned.
#pragma once
#include <cstdint>
#include "hqr_common.cuh"

namespace hqr {
namespace oz {

constexpr int kSlices = 8;         // slice storage per operand (the most a scheme uses)
constexpr int kN = 64;             // columns per update task (MMA N)
constexpr int kM = 128;            // rows per MMA (one TMEM lane per row)
constexpr int kKC = 16;            // K per BF16 MMA
constexpr int kGroups = 8;         // t-group accumulators: t = p + q in [2, 9] (1-based)
constexpr int kDC = 8;             // accumulator columns recombined per epilogue pass

// Digit schemes.  F (|F| < 2^55, the fixed-point form of an element relative
// to its row / column maximum) is written exactly as S digits of RHO bits:
// F = sum_{p=1..S} d_p 2^(RHO (S - p)), |d_p| <= 2^(RHO-1).  Slice products
// with p + q <= 9 are kept (8 t-groups, the whole TMEM); relative to
// rowmax * colmax the dropped ones weigh about 2^(-8 RHO):
//   Scheme8x7 (K <= 128): 8-bit digits, 7 slices, 34 products, drop < 2^-64;
//   Scheme7x8 (K <= 256): 7-bit digits, 8 slices, 36 products, drop < 2^-56.
// Exactness: a t-group holds <= S pairs of K products of |d d| <= 2^(2 RHO - 2),
// i.e. 7 * 128 * 2^14 < 2^24 and 8 * 256 * 2^12 = 2^23.
template <int RHO_, int S_, int SHIFT_HI_, int SHIFT_LO_, int EXP_BIAS_>
struct Scheme {
  static constexpr int RHO = RHO_;
  static constexpr int S = S_;
  static constexpr int SHIFT_HI = SHIFT_HI_;   // X = (hi << SHIFT_HI) + (lo >> SHIFT_LO)
  static constexpr int SHIFT_LO = SHIFT_LO_;
  static constexpr int EXP_BIAS = EXP_BIAS_;   // biased exponent of the scale = Ea + Eb - EXP_BIAS
};
using Scheme8x7 = Scheme<8, 7, 14, 18, 1073>;
using Scheme7x8 = Scheme<7, 8, 18, 10, 1072>;
constexpr int kAChunkBytes = kSlices * kM * kKC * 2;    // 32 KiB: all slices of one K chunk
constexpr int kBChunkBytes = kSlices * kN * kKC * 2;    // 16 KiB
constexpr int kSliceABytes = kM * kKC * 2;              // 4 KiB
constexpr int kSliceBBytes = kN * kKC * 2;              // 2 KiB
constexpr long long kWaitIters = 1LL << 26;             // bounded mbarrier waits

// Bytes of one prepared left operand (NB x NB) and of the three of a panel tile.
__host__ __device__ constexpr size_t operand_bytes(int NB) { return (size_t)NB * NB * kSlices * 2; }
__host__ __device__ constexpr size_t panel_slice_bytes(int NB) { return 3 * operand_bytes(NB); }

// ---------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
               : "memory");
}
// Wait for the phase with parity `parity`, bounded by kWaitNs of wall time
// and abandoned at once when the scheduler's error word is set; false then.
constexpr long long kWaitNs = 2000000000LL;
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, const unsigned* err) {
  const uint32_t a = smem_u32(b);
  const uint64_t t0 = global_ns();
  for (long long it = 0; it < kWaitIters; it++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if ((it & 255) == 255) {
      if (*((volatile const unsigned*)err) != 0u) return false;
      if ((long long)(global_ns() - t0) > kWaitNs) return false;
    }
  }
  return false;
}
__device__ __forceinline__ void tma_load_1d(void* dst_smem, const void* src_gmem, uint32_t bytes,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst_smem)),
      "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t* slot_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot_smem)),
               "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}
// K-major, no-swizzle shared-memory matrix descriptor (core matrices of
// 8 rows x 16 bytes; LBO = next core matrix along K, SBO = along M/N).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}
// Instruction descriptor: kind::f16, BF16 x BF16 -> FP32, K-major A and B.
__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t id,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(id), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
// 8 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                 "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------
// Slicing
// ---------------------------------------------------------------------------
__device__ __forceinline__ int biased_exp(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7ff);
}
// F = x * 2^(1077 - E) rounded to the nearest integer (|F| <= 2^55 when x's
// exponent <= E); subnormals and zeros give 0.  Rounding (not truncation)
// keeps the representation error of elements below the row / column maximum
// unbiased, so it does not accumulate coherently over successive updates.
__device__ __forceinline__ long long fixed_of(double x, int E) {
  const long long b = __double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e == 0) return 0;
  const long long m = (b & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
  const int sh = e - E + 2;
  long long F;
  if (sh >= 0)
    F = m << sh;
  else
    F = (sh > -60) ? ((m + (1LL << (-sh - 1))) >> (-sh)) : 0;
  return (b < 0) ? -F : F;
}
// Digits d_1..d_S of F (signed, round to nearest): F = sum d_p 2^(RHO (S - p)).
template <class SC>
__device__ __forceinline__ void digits(long long F, int* d) {
#pragma unroll
  for (int p = 0; p < SC::S - 1; p++) {
    const int u = SC::RHO * (SC::S - 1 - p);
    const long long dp = (F + (1LL << (u - 1))) >> u;
    d[p] = (int)dp;
    F -= dp << u;
  }
  d[SC::S - 1] = (int)F;
}
__device__ __forceinline__ uint32_t bf16_bits(int d) {
  return __float_as_uint((float)d) >> 16;    // exact: |d| <= 128 has <= 8 significant bits
}
// Byte offset of element (row, kk) (kk < 16) inside one K-major slice block
// of `rows` rows: core matrices [row/8][kk/8][8][16 bytes].
__device__ __forceinline__ int core_off(int row, int kk) {
  return ((row >> 3) * 2 + (kk >> 3)) * 128 + (row & 7) * 16 + (kk & 7) * 2;
}

// ---------------------------------------------------------------------------
// Per-CTA state of the engine (shared memory + TMEM)
// ---------------------------------------------------------------------------
struct Ctx {
  uint8_t* sA;          // 2 stages x kAChunkBytes
  uint8_t* sB;          // 2 stages x kBChunkBytes
  uint64_t* bar;        // [0,1] A full, [2,3] MMA done
  int* sEb;             // kN column exponents of the right operand
  double* sY;           // the right operand, staged: K x kN doubles, ld K + 1
  uint32_t tmem;        // base of the 512 TMEM columns
  uint32_t phase_a[2];  // phase parity per stage (kept identical in every thread)
  uint32_t phase_m[2];
  unsigned* err;        // scheduler error word
};

constexpr int kMaxK = 256;
constexpr int kYBytes = (kMaxK + 1) * kN * 8;
// Shared-memory bytes the engine needs.
constexpr int kSmemBytes = 2 * kAChunkBytes + 2 * kBChunkBytes + 64 + kN * 4 + 128 + kYBytes;

__device__ __forceinline__ void ctx_init(Ctx& c, uint8_t* base, uint32_t tmem, unsigned* err) {
  c.sA = base;
  c.sB = base + 2 * kAChunkBytes;
  c.bar = reinterpret_cast<uint64_t*>(base + 2 * kAChunkBytes + 2 * kBChunkBytes);
  c.sEb = reinterpret_cast<int*>(base + 2 * kAChunkBytes + 2 * kBChunkBytes + 64);
  c.sY = reinterpret_cast<double*>(base + 2 * kAChunkBytes + 2 * kBChunkBytes + 64 + kN * 4 + 128);
  c.tmem = tmem;
  c.err = err;
  if (threadIdx.x == 0) {
    for (int i = 0; i < 4; i++) mbar_init(c.bar + i, 1);
    mbar_fence_init();
  }
  for (int i = 0; i < 2; i++) {
    c.phase_a[i] = 0;
    c.phase_m[i] = 0;
  }
  __syncthreads();
}

__device__ __forceinline__ void set_err(const Ctx& c) {
  atomicOr(reinterpret_cast<int*>(c.err), kErrTimeout);
}

// Stage the kN-column right operand Y (K rows, ld ldy, global) in shared
// memory (ld K + 1: conflict-free column reads) and compute its column
// exponents (max biased exponent per column).
inline __device__ void stage_y(Ctx& c, const double* Y, int ldy, int K) {
  const int lds = K + 1;
  for (int e = threadIdx.x; e < K * kN / 2; e += kThreads) {
    const int col = (2 * e) / K, r = (2 * e) % K;               // K is even: pairs stay in a column
    const double2 v = __ldcg(reinterpret_cast<const double2*>(Y + (size_t)col * ldy + r));
    c.sY[col * lds + r] = v.x;
    c.sY[col * lds + r + 1] = v.y;
  }
  __syncthreads();
  const int col = threadIdx.x >> 2, part = threadIdx.x & 3;   // 4 threads per column
  int e = 0;
  if (col < kN) {
    const double* y = c.sY + col * lds;
    for (int r = part; r < K; r += 4) e = max(e, biased_exp(y[r]));
  }
  e = max(e, __shfl_xor_sync(0xffffffffu, e, 1));
  e = max(e, __shfl_xor_sync(0xffffffffu, e, 2));
  if (col < kN && part == 0) c.sEb[col] = e;
  __syncthreads();
}

// Slice rows [k0, k0+16) of the staged right operand (kN columns) into B stage `s`.
template <class SC>
__device__ __forceinline__ void slice_b_chunk(Ctx& c, int s, int K, int k0) {
  const int col = threadIdx.x >> 2, q = threadIdx.x & 3;   // 64 columns x 4 quads of 4 rows
  const int E = c.sEb[col];
  const double* y = c.sY + col * (K + 1) + k0 + 4 * q;
  int d[4][SC::S];
#pragma unroll
  for (int i = 0; i < 4; i++) digits<SC>(fixed_of(y[i], E), d[i]);
  uint8_t* stage = c.sB + s * kBChunkBytes;
  const int off = core_off(col, 4 * q);
#pragma unroll
  for (int p = 0; p < SC::S; p++) {
    uint2 w;
    w.x = bf16_bits(d[0][p]) | (bf16_bits(d[1][p]) << 16);
    w.y = bf16_bits(d[2][p]) | (bf16_bits(d[3][p]) << 16);
    *reinterpret_cast<uint2*>(stage + p * kSliceBBytes + off) = w;
  }
}

// One M-tile (128 rows) of an Ozaki product: the 8 t-group accumulators of
// X[mt] (prepared slices, K = K chunks [kc0, kc1)) times Y (kN columns, sliced
// here).  On return (true) the accumulators are final in TMEM.
template <class SC>
inline __device__ bool gemm_tile(Ctx& c, const uint8_t* Xprep, int KC, int mt, int kc0, int kc1) {
  const int K = KC * kKC;
  const uint32_t id = idesc_bf16(kM, kN);
  const uint64_t dA0 = sdesc(smem_u32(c.sA), 128, 256);
  const uint64_t dB0 = sdesc(smem_u32(c.sB), 128, 256);
  const uint8_t* src = Xprep + (size_t)mt * KC * kAChunkBytes;
  bool ok = true;
  // prologue: stage 0 <- chunk kc0
  if (threadIdx.x == 0) {
    mbar_expect_tx(c.bar + 0, kAChunkBytes);
    tma_load_1d(c.sA, src + (size_t)kc0 * kAChunkBytes, kAChunkBytes, c.bar + 0);
  }
  slice_b_chunk<SC>(c, 0, K, kc0 * kKC);
  for (int kc = kc0; kc < kc1; kc++) {
    const int s = (kc - kc0) & 1;
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      if (!mbar_wait(c.bar + s, c.phase_a[s], c.err)) ok = false;
      tc_fence_after();
      if (ok) {
        const uint64_t dA = dA0 + (uint64_t)((s * kAChunkBytes) >> 4);
        const uint64_t dB = dB0 + (uint64_t)((s * kBChunkBytes) >> 4);
        // pairs (p, q) (0-based) with p + q <= kGroups - 1; t-group ti = p + q;
        // the first product into each group in chunk kc0 overwrites it
#pragma unroll
        for (int p = 0; p < SC::S; p++) {
#pragma unroll
          for (int q = 0; q < SC::S && p + q < kGroups; q++) {
            const int first_p = (p + q) - (SC::S - 1) > 0 ? (p + q) - (SC::S - 1) : 0;
            const uint32_t acc = (kc > kc0 || p > first_p) ? 1u : 0u;
            mma_bf16(c.tmem + (uint32_t)((p + q) * kN), dA + (uint64_t)((p * kSliceABytes) >> 4),
                     dB + (uint64_t)((q * kSliceBBytes) >> 4), id, acc);
          }
        }
      }
      mma_commit(c.bar + 2 + s);
    }
    c.phase_a[s] ^= 1;
    if (kc + 1 < kc1) {
      const int s1 = s ^ 1;
      if (kc + 1 - kc0 >= 2) {   // stage s1 still feeds the MMAs of chunk kc-1
        if (!mbar_wait(c.bar + 2 + s1, c.phase_m[s1], c.err)) ok = false;
        c.phase_m[s1] ^= 1;
      }
      if (threadIdx.x == 0) {
        mbar_expect_tx(c.bar + s1, kAChunkBytes);
        tma_load_1d(c.sA + s1 * kAChunkBytes, src + (size_t)(kc + 1) * kAChunkBytes, kAChunkBytes,
                    c.bar + s1);
      }
      slice_b_chunk<SC>(c, s1, K, (kc + 1) * kKC);
    }
  }
  // drain the (up to two) outstanding commits
  const int n = kc1 - kc0;
  for (int k = (n >= 2 ? n - 2 : 0); k < n; k++) {
    const int s = k & 1;
    if (!mbar_wait(c.bar + 2 + s, c.phase_m[s], c.err)) ok = false;
    c.phase_m[s] ^= 1;
  }
  tc_fence_after();
  ok = __syncthreads_and(ok) != 0;   // uniform across the CTA
  if (!ok && threadIdx.x == 0) set_err(c);
  return ok;
}

// Epilogue modes.
enum Epi : int {
  kEpiStoreAdd = 0,   // out = addend (or 0) + R
  kEpiStoreSub = 1,   // out = R; top -= R (when top != nullptr)
  kEpiSubInto = 2,    // tgt -= R
};

// X * 2^(se - 1023) as binary64, rounded to nearest even, built with integer
// operations from the IEEE 754 encoding (normalise |X|, round to 53 bits,
// add the exponent).  The FP64 units of this part are scarce; the epilogue
// keeps them for the one addition per element.  Falls back to FP64
// arithmetic when the result is not a normal number.
__device__ __forceinline__ double scaled_i64(long long X, int se) {
  if (X == 0) return 0.0;
  const unsigned long long sign = (X < 0) ? (1ULL << 63) : 0ULL;
  unsigned long long u = (X < 0) ? 0ULL - (unsigned long long)X : (unsigned long long)X;
  const int lz = __clzll((long long)u);
  u <<= lz;                                              // leading one at bit 63
  unsigned long long m = u >> 11;                        // 53 significant bits
  const unsigned rem = (unsigned)u & 0x7FFu;
  m += (rem > 0x400u || (rem == 0x400u && (m & 1ULL))) ? 1ULL : 0ULL;
  const int e = se + 63 - lz;                            // biased exponent before a carry
  // m carries its leading one into the exponent field (and a rounding carry
  // to 2^53 bumps the exponent once more, with a zero fraction)
  const unsigned long long bits = ((unsigned long long)(e - 1) << 52) + m;
  const int ef = (int)(bits >> 52);
  if (e < 1 || ef > 2046) {
    const double scale = (se > 0 && se < 2047) ? __longlong_as_double((long long)se << 52)
                                               : ldexp(1.0, se - 1023);
    return (double)X * scale;
  }
  return __longlong_as_double((long long)(sign | bits));
}

// Recombine the 8 t-group accumulators of M-tile mt into FP64 and apply the
// epilogue.  Warp w handles rows 32*(w%4).., columns 32*(w/4)..+31.
template <class SC>
inline __device__ void drain(Ctx& c, int mt, const int* Ea, int mode, double* out, int ldo,
                             const double* addend, int lda, double* top, int ldt) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = mt * kM + 32 * (w & 3) + lane;
  const int cb = 32 * (w >> 2);
  const int ea = __ldcg(Ea + row);
  const uint32_t lane_addr = c.tmem + ((uint32_t)(32 * (w & 3)) << 16);
  // the memory operand of each mode: addend, top, or the target itself
  const double* msrc = (mode == kEpiStoreAdd) ? addend : (mode == kEpiStoreSub) ? top : out;
  const int mld = (mode == kEpiStoreAdd) ? lda : (mode == kEpiStoreSub) ? ldt : ldo;
  for (int pass = 0; pass < 32 / kDC; pass++) {
    const int c0 = cb + kDC * pass;
    // issue the memory loads before the TMEM reads so they overlap
    double mem[kDC];
#pragma unroll
    for (int i = 0; i < kDC; i++) mem[i] = msrc ? ldg_cg(msrc + row + (size_t)(c0 + i) * mld) : 0.0;
    long long hi[kDC], lo[kDC];
#pragma unroll
    for (int i = 0; i < kDC; i++) hi[i] = lo[i] = 0;
#pragma unroll
    for (int t = 0; t < kGroups; t++) {
      float v[kDC];
      tmem_ld8(lane_addr + (uint32_t)(t * kN + c0), v);
#pragma unroll
      for (int i = 0; i < kDC; i++) {
        const long long g = (long long)__float2int_rn(v[i]);
        if (t < 4)
          hi[i] = (hi[i] << SC::RHO) + g;
        else
          lo[i] = (lo[i] << SC::RHO) + g;
      }
    }
#pragma unroll
    for (int i = 0; i < kDC; i++) {
      const int col = c0 + i;
      const long long X =
          (hi[i] << SC::SHIFT_HI) + ((lo[i] + (1LL << (SC::SHIFT_LO - 1))) >> SC::SHIFT_LO);
      const int eb = c.sEb[col];
      const int se = ea + eb - SC::EXP_BIAS;   // biased exponent of the scale of X
      const double r = (ea > 0 && eb > 0) ? scaled_i64(X, se) : 0.0;
      const size_t o = (size_t)col;
      if (mode == kEpiStoreAdd) {
        stg_cg(out + row + o * ldo, mem[i] + r);
      } else if (mode == kEpiStoreSub) {
        stg_cg(out + row + o * ldo, r);
        if (top) stg_cg(top + row + o * ldt, mem[i] - r);
      } else {
        stg_cg(out + row + o * ldo, mem[i] - r);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
}

// One full Ozaki product for an NB-row left operand (all M-tiles).
// tri: 0 dense, 1 X lower triangular (rows r need K <= r), 2 X upper
// triangular (rows r need K >= r).
template <class SC>
inline __device__ bool product(Ctx& c, int NB, const uint8_t* Xprep, const int* Ea, int tri,
                               const double* Y, int ldy, int mode, double* out, int ldo,
                               const double* addend, int lda, double* top, int ldt) {
  const int KC = NB / kKC;
  stage_y(c, Y, ldy, NB);
  for (int mt = 0; mt < NB / kM; mt++) {
    int kc0 = 0, kc1 = KC;
    if (tri == 1) kc1 = min(KC, (mt + 1) * kM / kKC);
    if (tri == 2) kc0 = mt * kM / kKC;
    if (!gemm_tile<SC>(c, Xprep, KC, mt, kc0, kc1)) return false;
    drain<SC>(c, mt, Ea, mode, out, ldo, addend, lda, top, ldt);
  }
  return true;
}

// ---------------------------------------------------------------------------
// Preparation of a panel tile's left operands (once per panel tile)
// ---------------------------------------------------------------------------
// Slice an NB x NB left operand X into the [mt][kc][slice][core layout]
// order; X(r, k) = src[r*rs + k*ks]; Ea[r] = max biased exponent of row r.
template <class SC>
inline __device__ void prep_operand(const double* src, int rs, int ks, int NB, uint8_t* dst, int* Ea,
                                    int kind_unit_lower) {
  // row exponents
  for (int r = threadIdx.x; r < NB; r += kThreads) {
    int e = 0;
    for (int k = 0; k < NB; k++) {
      double x = ldg_cg(src + (size_t)r * rs + (size_t)k * ks);
      if (kind_unit_lower == 1) x = (r > k) ? x : (r == k ? 1.0 : 0.0);        // V (unit lower)
      if (kind_unit_lower == 2) x = (k > r) ? x : (k == r ? 1.0 : 0.0);        // V^T of unit lower V
      if (kind_unit_lower == 3) x = (k <= r) ? x : 0.0;                          // T^T (lower)
      e = max(e, biased_exp(x));
    }
    Ea[r] = e;
  }
  __syncthreads();
  const int KC = NB / kKC;
  // one thread per (row, k-quad)
  const int quads = NB * NB / 4;
  for (int qd = threadIdx.x; qd < quads; qd += kThreads) {
    const int r = qd % NB;
    const int k4 = (qd / NB) * 4;
    const int E = Ea[r];
    int d[4][SC::S];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int k = k4 + i;
      double x = ldg_cg(src + (size_t)r * rs + (size_t)k * ks);
      if (kind_unit_lower == 1) x = (r > k) ? x : (r == k ? 1.0 : 0.0);
      if (kind_unit_lower == 2) x = (k > r) ? x : (k == r ? 1.0 : 0.0);
      if (kind_unit_lower == 3) x = (k <= r) ? x : 0.0;
      digits<SC>(fixed_of(x, E), d[i]);
    }
    const int mt = r / kM, kc = k4 / kKC;
    uint8_t* blk = dst + ((size_t)mt * KC + kc) * kAChunkBytes;
    const int off = core_off(r % kM, k4 % kKC);
#pragma unroll
    for (int p = 0; p < SC::S; p++) {
      uint2 w;
      w.x = bf16_bits(d[0][p]) | (bf16_bits(d[1][p]) << 16);
      w.y = bf16_bits(d[2][p]) | (bf16_bits(d[3][p]) << 16);
      *reinterpret_cast<uint2*>(blk + p * kSliceABytes + off) = w;
    }
  }
  __syncthreads();
}

}  // namespace oz
}  // namespace hqr
