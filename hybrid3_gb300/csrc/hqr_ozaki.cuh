// hqr_ozaki.cuh -- split-precision products on the 5th-generation tensor
// cores (tcgen05, TMEM accumulators, bulk-TMA operand staging).
//
// Every product is X Y with a 128 x 128 left operand X (a panel tile's V^T,
// T^T or V) and a 128 x 64 right operand Y (a column block of a trailing
// tile), computed as an Ozaki-style sum of exact slice products (Ozaki,
// Ogita, Oishi, Rump, "Error-free transformations of matrix multiplication by
// using fast routines of matrix multiplication and its applications", Numer.
// Algorithms 59, 2012):
//
//   * every row of X (and every column of Y) is scaled by the power of two of
//     its largest element and written as a fixed-point integer F, |F| < 2^62,
//     so an element 2^-9 of its row maximum still keeps 53 bits;
//   * F is split into kS = 8 signed digits of kRho = 8 bits, |d_0| <= 64,
//     |d_p| <= 128, F = sum_p d_p 2^(8 (7 - p)); every digit is an exact BF16
//     value;
//   * the slice products X_p Y_q with p + q <= 7 (0-based; 36 of the 64) are
//     exact on the tensor cores: |d_x d_y| <= 2^14, a K = 128 sum stays below
//     2^21, and the <= 8 products sharing t = p + q (weight 2^(-8t)) are
//     accumulated in one FP32 TMEM accumulator, < 7 * 2^21 < 2^24 (the two
//     products with the top digit are at most 2^13);
//   * the 8 t-group accumulators (8 x 64 TMEM columns = the whole TMEM) are
//     recombined exactly in 64-bit integers (two Horner chains in base 2^8,
//     V = hi 2^32 + lo, up to 77 bits), shifted right only as far as V's bit
//     length requires to fit 63 bits, rounding to odd, and converted to FP64
//     with integer operations: the result is V correctly rounded, once.  The
//     dropped products weigh < 2^-58 of rowmax(X) * colmax(Y) * K.
//
// The left operands are sliced once per panel tile into HBM, already in the
// tcgen05 K-major core-matrix layout, so each 16-deep K chunk of all 8 slices
// arrives with one 32 KiB bulk TMA copy.  The right operand lives in shared
// memory (staged from HBM for the first product of an update, written there
// by the previous product's epilogue otherwise) and is sliced chunk by chunk
// into a double-buffered stage while the MMAs of the previous chunk run.
// MMAs are issued by one thread (M = 128, N = 64, K = 16, BF16 x BF16 ->
// FP32).  Every mbarrier wait is bounded; on time-out the error word is set
// and the task is abandoned.
#pragma once
#include <cstdint>
#include "hqr_common.cuh"

namespace hqr {
namespace oz {

constexpr int kK = 128;            // the tile order: K (and M) of every product
constexpr int kN = 64;             // columns of the right operand (MMA N)
constexpr int kM = 128;            // rows per MMA (one TMEM lane per row)
constexpr int kKC = 16;            // K per BF16 MMA
constexpr int kChunks = kK / kKC;  // 8 K chunks per product
constexpr int kRho = 8;            // bits per digit
constexpr int kS = 8;              // digits (slices) per element
constexpr int kGroups = 8;         // t-group accumulators: t = p + q in [0, 7]
constexpr int kExpBias = 1089;     // biased exponent of the scale of V = hi 2^32 + lo: Ea + Eb - kExpBias
constexpr int kDC = 8;             // accumulator columns recombined per epilogue pass (tmem_ld_groups)
constexpr int kLdY = kK + 2;       // leading dimension of the staged right operand (16-byte columns)
constexpr int kLdT = kK + 1;       // leading dimension of a staged 128 x 128 tile
constexpr int kSliceABytes = kM * kKC * 2;              // 4 KiB
constexpr int kSliceBBytes = kN * kKC * 2;              // 2 KiB
constexpr int kAChunkBytes = kS * kSliceABytes;         // 32 KiB: all slices of one K chunk
constexpr int kBChunkBytes = kS * kSliceBBytes;         // 16 KiB
constexpr long long kWaitIters = 1LL << 26;             // bounded mbarrier waits

// Bytes of one prepared left operand and of the kSlots of a panel tile
// (V^T, T^T, V, and T for applying the reflector itself).
constexpr int kSlots = 4;
__host__ __device__ constexpr size_t operand_bytes() { return (size_t)kK * kK * kS * 2; }
__host__ __device__ constexpr size_t panel_slice_bytes() { return kSlots * operand_bytes(); }

// Pipeline depth: A chunks (bulk TMA) and sliced B chunks in flight.
constexpr int kAStages = 3;
constexpr int kBStages = 4;
// done barriers: one per chunk in flight on either ring, so that no two
// chunks a wait may still refer to share a barrier (parity waits stay exact)
constexpr int kDoneStages = kAStages > kBStages ? kAStages : kBStages;
constexpr int kSlicerWarps = kWarps - 1;   // warp 0 issues the copies and the MMAs
// Barriers: a_full[kAStages] (TMA bytes), b_full[kBStages] (one arrival per
// slicer warp), done[kDoneStages] (tcgen05.commit of one chunk's MMAs).
constexpr int kBarAFull = 0, kBarBFull = kAStages, kBarDone = kAStages + kBStages;
constexpr int kNumBars = kAStages + kBStages + kDoneStages;
// Shared-memory map of the engine.
constexpr int kOffB = kAStages * kAChunkBytes;
constexpr int kOffBar = kOffB + kBStages * kBChunkBytes;
constexpr int kOffEb = kOffBar + 128;
constexpr int kOffY = kOffEb + 2 * kN * 4;
constexpr int kSmemBytes = kOffY + kLdY * kN * 8;
static_assert(kNumBars * 8 <= 128, "barrier area");
static_assert(kOffY % 16 == 0, "staged operand alignment");

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
// 16-byte asynchronous global -> shared copies (L2 only), all in flight
// until cp_async_wait_all.
__device__ __forceinline__ void cp_async16(void* dst_smem, const void* src_gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst_smem)), "l"(src_gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Orders this thread's generic-proxy global writes (prepared slices) with
// bulk-TMA reads of them (async proxy).
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
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
// Columns c..c+7 of all 8 t-group accumulators (group t at column t * kN + c)
// of this thread's TMEM lane: eight loads, one wait.  The outputs are
// early-clobber: a load must not overwrite the address of a later one.
__device__ __forceinline__ void tmem_ld_groups(uint32_t taddr, uint32_t (&r)[8][8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%64];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%65];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16,%17,%18,%19,%20,%21,%22,%23}, [%66];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%24,%25,%26,%27,%28,%29,%30,%31}, [%67];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%32,%33,%34,%35,%36,%37,%38,%39}, [%68];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%40,%41,%42,%43,%44,%45,%46,%47}, [%69];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%48,%49,%50,%51,%52,%53,%54,%55}, [%70];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%56,%57,%58,%59,%60,%61,%62,%63}, [%71];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=&r"(r[0][0]), "=&r"(r[0][1]), "=&r"(r[0][2]), "=&r"(r[0][3]), "=&r"(r[0][4]), "=&r"(r[0][5]), "=&r"(r[0][6]), "=&r"(r[0][7]), "=&r"(r[1][0]), "=&r"(r[1][1]), "=&r"(r[1][2]), "=&r"(r[1][3]), "=&r"(r[1][4]), "=&r"(r[1][5]), "=&r"(r[1][6]), "=&r"(r[1][7]), "=&r"(r[2][0]), "=&r"(r[2][1]), "=&r"(r[2][2]), "=&r"(r[2][3]), "=&r"(r[2][4]), "=&r"(r[2][5]), "=&r"(r[2][6]), "=&r"(r[2][7]), "=&r"(r[3][0]), "=&r"(r[3][1]), "=&r"(r[3][2]), "=&r"(r[3][3]), "=&r"(r[3][4]), "=&r"(r[3][5]), "=&r"(r[3][6]), "=&r"(r[3][7]), "=&r"(r[4][0]), "=&r"(r[4][1]), "=&r"(r[4][2]), "=&r"(r[4][3]), "=&r"(r[4][4]), "=&r"(r[4][5]), "=&r"(r[4][6]), "=&r"(r[4][7]), "=&r"(r[5][0]), "=&r"(r[5][1]), "=&r"(r[5][2]), "=&r"(r[5][3]), "=&r"(r[5][4]), "=&r"(r[5][5]), "=&r"(r[5][6]), "=&r"(r[5][7]), "=&r"(r[6][0]), "=&r"(r[6][1]), "=&r"(r[6][2]), "=&r"(r[6][3]), "=&r"(r[6][4]), "=&r"(r[6][5]), "=&r"(r[6][6]), "=&r"(r[6][7]), "=&r"(r[7][0]), "=&r"(r[7][1]), "=&r"(r[7][2]), "=&r"(r[7][3]), "=&r"(r[7][4]), "=&r"(r[7][5]), "=&r"(r[7][6]), "=&r"(r[7][7])
      : "r"(taddr), "r"(taddr + 1 * kN), "r"(taddr + 2 * kN), "r"(taddr + 3 * kN), "r"(taddr + 4 * kN),
        "r"(taddr + 5 * kN), "r"(taddr + 6 * kN), "r"(taddr + 7 * kN)
      : "memory");
}

// The first four t-group accumulators only (the products of weight t <= 3).
__device__ __forceinline__ void tmem_ld_groups4(uint32_t taddr, uint32_t (&r)[8][8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%32];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%33];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16,%17,%18,%19,%20,%21,%22,%23}, [%34];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%24,%25,%26,%27,%28,%29,%30,%31}, [%35];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=&r"(r[0][0]), "=&r"(r[0][1]), "=&r"(r[0][2]), "=&r"(r[0][3]), "=&r"(r[0][4]), "=&r"(r[0][5]),
        "=&r"(r[0][6]), "=&r"(r[0][7]), "=&r"(r[1][0]), "=&r"(r[1][1]), "=&r"(r[1][2]), "=&r"(r[1][3]),
        "=&r"(r[1][4]), "=&r"(r[1][5]), "=&r"(r[1][6]), "=&r"(r[1][7]), "=&r"(r[2][0]), "=&r"(r[2][1]),
        "=&r"(r[2][2]), "=&r"(r[2][3]), "=&r"(r[2][4]), "=&r"(r[2][5]), "=&r"(r[2][6]), "=&r"(r[2][7]),
        "=&r"(r[3][0]), "=&r"(r[3][1]), "=&r"(r[3][2]), "=&r"(r[3][3]), "=&r"(r[3][4]), "=&r"(r[3][5]),
        "=&r"(r[3][6]), "=&r"(r[3][7])
      : "r"(taddr), "r"(taddr + 1 * kN), "r"(taddr + 2 * kN), "r"(taddr + 3 * kN)
      : "memory");
#pragma unroll
  for (int t = 4; t < 8; t++)
#pragma unroll
    for (int i = 0; i < 8; i++) r[t][i] = 0u;   // FP32 zero: the dropped groups
}

// ---------------------------------------------------------------------------
// Slicing
// ---------------------------------------------------------------------------
__device__ __forceinline__ int biased_exp(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7ff);
}
// F = x * 2^(1084 - E) rounded to the nearest integer, halves away from zero
// (|F| < 2^62 when x's exponent e <= E); subnormals and zeros give 0.
// Rounding (not truncation) keeps the representation error of elements below
// the row / column maximum unbiased, so it does not accumulate coherently over
// successive updates.
__device__ __forceinline__ long long fixed_of(double x, int E) {
  const long long b = __double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  const int k = E - e;   // >= 0: E is the maximum exponent of the row / column
  if (e == 0 || k > 63) return 0;
  const unsigned long long t = ((unsigned long long)(b & 0xFFFFFFFFFFFFFLL) | (1ULL << 52)) << 9;
  const unsigned long long F = (k == 0) ? t : (((t >> (k - 1)) + 1ULL) >> 1);
  return (b < 0) ? -(long long)F : (long long)F;
}
// Balanced base-256 digits d_0..d_7 of F (|F| < 2^62) as exact floats:
// F = sum d_p 2^(8 (7 - p)), d_1..d_7 in [-128, 127], d_0 in [-64, 64].
// Adding 128 at each of the seven low byte positions, G = F + 0x80808080808080
// (no overflow: |G| < 2^63), lets the carries do the balancing: byte j of G is
// d_(7-j) + 128 (j < 7) and G >> 56 is d_0.  The float of byte b - 128 is
// (2^23 + b) - (2^23 + 128), with 2^23 + b assembled by one byte permute:
// exact, no conversion unit.
__device__ __forceinline__ void digits(long long F, float* d) {
  const long long G = F + 0x0080808080808080LL;
  const uint32_t lo = (uint32_t)G, hi = (uint32_t)((unsigned long long)G >> 32);
#pragma unroll
  for (int j = 0; j < kS - 1; j++) {
    const uint32_t bits = __byte_perm(j < 4 ? lo : hi, 0x4B000000u, 0x7440u | (uint32_t)(j & 3));
    d[kS - 1 - j] = __uint_as_float(bits) - 8388736.0f;
  }
  d[0] = (float)(int)(G >> 56);
}
// Two BF16 digits in one word: the upper halves of their (exact) FP32 images.
__device__ __forceinline__ uint32_t bf16x2(float d0, float d1) {
  return __byte_perm(__float_as_uint(d0), __float_as_uint(d1), 0x7632);
}
// Byte offset of element (row, kk) (kk < 16) inside one K-major slice block:
// core matrices [row/8][kk/8][8][16 bytes].
__device__ __forceinline__ int core_off(int row, int kk) {
  return ((row >> 3) * 2 + (kk >> 3)) * 128 + (row & 7) * 16 + (kk & 7) * 2;
}

// ---------------------------------------------------------------------------
// Per-CTA state of the engine (shared memory + TMEM)
// ---------------------------------------------------------------------------
struct Ctx {
  uint8_t* sA;          // kAStages x kAChunkBytes
  uint8_t* sB;          // kBStages x kBChunkBytes
  uint64_t* bar;        // kNumBars mbarriers (kBarAFull, kBarBFull, kBarDone)
  int* sEb;             // 2 x kN column exponents of the right operand
  double* sY;           // the right operand: kK x kN doubles, ld kLdY
  uint32_t tmem;        // base of the 512 TMEM columns
  int n;                // K chunks consumed so far in this task (same in every thread)
  int na;               // K chunks whose A copy has been issued (thread 0 only)
  int yb;               // which half of sEb describes sY
  unsigned* err;        // scheduler error word
};

__device__ __forceinline__ void ctx_init(Ctx& c, uint8_t* base, uint32_t tmem, unsigned* err) {
  c.sA = base;
  c.sB = base + kOffB;
  c.bar = reinterpret_cast<uint64_t*>(base + kOffBar);
  c.sEb = reinterpret_cast<int*>(base + kOffEb);
  c.sY = reinterpret_cast<double*>(base + kOffY);
  c.tmem = tmem;
  c.err = err;
  c.n = 0;
  c.na = 0;
  c.yb = 0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kNumBars; i++)
      mbar_init(c.bar + i, (i >= kBarBFull && i < kBarDone) ? kSlicerWarps : 1);
    mbar_fence_init();
  }
  __syncthreads();
}
// After the last product of a task: every copy and MMA has completed; the
// barriers are invalidated so the next task may reuse their shared memory.
__device__ __forceinline__ void ctx_release(Ctx& c) {
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 0; i < kNumBars; i++)
      asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(c.bar + i)) : "memory");
  __syncthreads();
}

__device__ __forceinline__ void set_err(const Ctx& c) {
  atomicOr(reinterpret_cast<int*>(c.err), kErrTimeout);
}

// Column exponents (max biased exponent) of the staged right operand into
// sEb[c.yb]; with Y2 (shared, kK x kN, ld kK) the exponents span both, for a
// right operand whose second half is reloaded into sY during the product.
__device__ __forceinline__ void y_exponents(Ctx& c, const double* Y2 = nullptr) {
  // warp w takes columns w * kColsW ..; its lanes read consecutive rows
  // (conflict-free), one warp max-reduction per column
  constexpr int kColsW = kN / kWarps;
  static_assert(kColsW * kWarps == kN, "columns per warp");
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll 2
  for (int cc = 0; cc < kColsW; cc++) {
    const int col = w * kColsW + cc;
    const double* y = c.sY + col * kLdY;
    int e = 0;
#pragma unroll
    for (int r = lane; r < kK; r += 32) e = max(e, biased_exp(y[r]));
    if (Y2) {
      const double* y2 = Y2 + col * kK;
#pragma unroll
      for (int r = lane; r < kK; r += 32) e = max(e, biased_exp(y2[r]));
    }
    e = (int)__reduce_max_sync(0xffffffffu, (unsigned)e);
    if (lane == 0) c.sEb[c.yb * kN + col] = e;
  }
  __syncthreads();
}

// Stage the right operand Y (kK x kN, column-major, ld ldy, global) in
// shared memory.  col0 >= 0: Y is the column block starting at column col0 of
// a unit-lower V (zero above the diagonal, one on it), or with `upper` of an
// upper-triangular V (zero below the diagonal).
// A kK x kN column block (global, column stride ld doubles, 16-byte aligned
// columns) into shared memory at dst (column stride ldd) with asynchronous
// copies issued by threads t0, t0 + nt, ... (not waited for).
__device__ __forceinline__ void cp_async_block(double* dst, int ldd, const double* src, int ld, int t0, int nt) {
  for (int e = t0; e < kK * kN / 2; e += nt) {
    const int col = e / (kK / 2), r = 2 * (e % (kK / 2));
    cp_async16(dst + col * ldd + r, src + (size_t)col * ld + r);
  }
}

__device__ __forceinline__ void stage_y(Ctx& c, const double* Y, int ldy, int col0, bool upper = false,
                                        const double* Yjoint = nullptr) {
  static_assert(kK * kN / 2 % kThreads == 0, "staging loop");
  static_assert(kBStages * kBChunkBytes == kK * kN * 8, "the B ring holds one column block");
  if (col0 < 0) {
    // unmasked: every copy in flight at once; Yjoint (ld kK) goes to the B
    // ring, idle until the product starts, for its column exponents
    cp_async_block(c.sY, kLdY, Y, ldy, threadIdx.x, kThreads);
    double* sJ = reinterpret_cast<double*>(c.sB);
    if (Yjoint) cp_async_block(sJ, kK, Yjoint, kK, threadIdx.x, kThreads);
    cp_async_wait_all();
    __syncthreads();
    y_exponents(c, Yjoint ? sJ : nullptr);
    return;
  }
  constexpr int kIter = kK * kN / 2 / kThreads;   // pairs per thread
#pragma unroll 4
  for (int it = 0; it < kIter; it++) {
    const int e = threadIdx.x + it * kThreads;
    const int col = e / (kK / 2), r = 2 * (e % (kK / 2));
    double2 v = __ldcg(reinterpret_cast<const double2*>(Y + (size_t)col * ldy + r));
    if (col0 >= 0) {
      const int gc = col0 + col;
      if (upper) {
        v.x = (r <= gc) ? v.x : 0.0;
        v.y = (r + 1 <= gc) ? v.y : 0.0;
      } else {
        v.x = (r > gc) ? v.x : (r == gc ? 1.0 : 0.0);
        v.y = (r + 1 > gc) ? v.y : (r + 1 == gc ? 1.0 : 0.0);
      }
    }
    *reinterpret_cast<double2*>(c.sY + col * kLdY + r) = v;
  }
  __syncthreads();
  y_exponents(c, Yjoint);
}

// Element masks of a panel tile's reflectors V (row i, column j of the tile).
enum Kind : int {
  kDense = 0,
  kUnitLower = 1,    // V of a GEQRT tile: zero above the diagonal, one on it
  kUnitUpper = 2,    // V^T of a GEQRT tile
  kUpperIncl = 3,    // V of a TT merge: upper triangle with the diagonal, zero below
  kLowerIncl = 4,    // V^T of a TT merge
};
__device__ __forceinline__ double mask_v(double v, int i, int j, int kind) {
  if (kind == kUnitLower) return (i > j) ? v : (i == j ? 1.0 : 0.0);
  if (kind == kUpperIncl) return (i <= j) ? v : 0.0;
  return v;
}

// Stage the column block col0.. of V^T as the right operand: Y(r, cc) =
// V(col0 + cc, r), V a 128 x 128 tile (global, ld kK) with mask `kind`.
__device__ __forceinline__ void stage_yt(Ctx& c, const double* V, int col0, int kind) {
  constexpr int kIter = kK * kN / kThreads;
#pragma unroll 4
  for (int it = 0; it < kIter; it++) {
    const int e = threadIdx.x + it * kThreads;
    const int cc = e % kN, r = e / kN;   // consecutive threads read consecutive rows of V's column r
    const int i = col0 + cc;
    c.sY[cc * kLdY + r] = mask_v(__ldcg(V + (size_t)i + (size_t)r * kK), i, r, kind);
  }
  __syncthreads();
  y_exponents(c);
}

// Slice quad g (column g / 4 of 64, rows k0 + 4 (g % 4) .. +3) of the staged
// right operand into B stage `s` (digit planes 0..G-1).
template <int G = kGroups>
__device__ __forceinline__ void slice_b_quad(Ctx& c, uint8_t* stage, int g, int k0) {
  const int col = g >> 2, q = g & 3;
  const int E = c.sEb[c.yb * kN + col];
  // two 16-byte loads: conflict-free (a quarter warp covers all 8 16-byte bank groups)
  const double2* y = reinterpret_cast<const double2*>(c.sY + col * kLdY + k0 + 4 * q);
  const double2 y01 = y[0], y23 = y[1];
  float d[4][kS];
  digits(fixed_of(y01.x, E), d[0]);
  digits(fixed_of(y01.y, E), d[1]);
  digits(fixed_of(y23.x, E), d[2]);
  digits(fixed_of(y23.y, E), d[3]);
  const int off = core_off(col, 4 * q);
#pragma unroll
  for (int p = 0; p < G; p++) {
    uint2 w;
    w.x = bf16x2(d[0][p], d[1][p]);
    w.y = bf16x2(d[2][p], d[3][p]);
    *reinterpret_cast<uint2*>(stage + p * kSliceBBytes + off) = w;
  }
}

__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
// Wait for the completion of task chunk n on barrier array `base` of `stages`.
__device__ __forceinline__ bool wait_chunk(const Ctx& c, int base, int stages, int n) {
  return mbar_wait(c.bar + base + n % stages, (uint32_t)((n / stages) & 1), c.err);
}
// Chunk `chunk` of X into A stage n: its digit planes 0..G-1 (the first G x 4
// KiB of the chunk).
template <int G = kGroups>
__device__ __forceinline__ void issue_a(Ctx& c, const uint8_t* X, int chunk, int n) {
  uint64_t* b = c.bar + kBarAFull + n % kAStages;
  mbar_expect_tx(b, G * kSliceABytes);
  tma_load_1d(c.sA + (n % kAStages) * kAChunkBytes, X + (size_t)chunk * kAChunkBytes, G * kSliceABytes, b);
}

// Issue the bulk copies of the first chunks of the next product's left
// operand X (thread 0), e.g. before the right operand is staged.
template <int G = kGroups>
__device__ __forceinline__ void prefetch(Ctx& c, const uint8_t* X) {
  if (threadIdx.x == 0) {
    fence_proxy_async_global();
    for (; c.na < c.n + kAStages; c.na++) issue_a<G>(c, X, c.na - c.n, c.na);
  }
}

// Barrier among the slicer warps only (warp 0 keeps issuing MMAs).
__device__ __forceinline__ void slicer_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(kSlicerWarps * 32) : "memory");
}

// The 8 t-group accumulators of X (prepared slices) times the staged right
// operand; Xnext (or nullptr): the left operand of the next product, whose
// first chunks are fetched as soon as their stages are free.  Warp 0, one
// thread: bulk copies of A and the MMAs; warps 1..7: slicing of B, up to
// kBStages chunks ahead of the MMAs.  On return (true) the accumulators are
// final in TMEM.  G < 8: only the pairs of weight p + q < G (accumulators
// 0..G-1; the others are left as they are).  nch: K chunks (8, or 16 for a
// K = 256 product whose right operand's second half, `reload` (global, kK x
// kN, ld kK), replaces the staged one once the slicers are past chunk 7; the
// column exponents must already span both halves).
template <int G = kGroups>
inline __device__ bool gemm(Ctx& c, const uint8_t* X, const uint8_t* Xnext, int nch = kChunks,
                            const double* reload = nullptr) {
  static_assert(G >= 1 && G <= kGroups, "t-groups");
  const int n0 = c.n;
  bool ok = true;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) {
    if (lane == 0) {
      const uint32_t id = idesc_bf16(kM, kN);
      const uint64_t dA0 = sdesc(smem_u32(c.sA), 128, 256);
      const uint64_t dB0 = sdesc(smem_u32(c.sB), 128, 256);
      fence_proxy_async_global();
      // chunks of this product not prefetched yet (stages free: every earlier MMA is done)
      for (; c.na < n0 + kAStages; c.na++) issue_a<G>(c, X, c.na - n0, c.na);
      for (int j = 0; j < nch && ok; j++) {
        const int n = n0 + j;
        if (!wait_chunk(c, kBarAFull, kAStages, n) || !wait_chunk(c, kBarBFull, kBStages, n)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint64_t dA = dA0 + (uint64_t)(((n % kAStages) * kAChunkBytes) >> 4);
        const uint64_t dB = dB0 + (uint64_t)(((n % kBStages) * kBChunkBytes) >> 4);
        // pairs (p, q) with p + q <= G - 1 into t-group p + q; the first
        // product into each group in chunk 0 overwrites it
#pragma unroll
        for (int p = 0; p < kS && p < G; p++) {
#pragma unroll
          for (int q = 0; q < kS && p + q < G; q++) {
            const int first_p = (p + q) - (kS - 1) > 0 ? (p + q) - (kS - 1) : 0;
            const uint32_t acc = (j > 0 || p > first_p) ? 1u : 0u;
            mma_bf16(c.tmem + (uint32_t)((p + q) * kN), dA + (uint64_t)((p * kSliceABytes) >> 4),
                     dB + (uint64_t)((q * kSliceBBytes) >> 4), id, acc);
          }
        }
        mma_commit(c.bar + kBarDone + n % kDoneStages);
        // refill the A stage of chunk n - 1 with chunk n - 1 + kAStages once its MMAs are done
        if (j >= 1 && j + kAStages - 1 < nch) {
          if (!wait_chunk(c, kBarDone, kDoneStages, n - 1)) {
            ok = false;
            break;
          }
          issue_a<G>(c, X, j + kAStages - 1, n + kAStages - 1);
          c.na = n + kAStages;
        }
      }
      // prefetch the next product's first chunks into the stages of the last kAStages
      if (ok && Xnext) {
        for (int j = 0; j < kAStages; j++) {
          if (!wait_chunk(c, kBarDone, kDoneStages, n0 + nch - kAStages + j)) {
            ok = false;
            break;
          }
          issue_a<G>(c, Xnext, j, n0 + nch + j);
        }
        if (ok) c.na = n0 + nch + kAStages;
      }
    }
    __syncwarp();
  } else {
    // slicer thread ts owns quads ts, ts + 224, ... of the product's nch x 256;
    // every slicer thread passes every loop step and the reload barriers, so
    // a failed wait (ok false, warp-uniform) skips work but never a barrier
    const int ts = threadIdx.x - 32;
    constexpr int kStride = kSlicerWarps * 32;
    int g = ts;
    for (int j = 0; j < nch; j++) {
      const int n = n0 + j;
      if (ok && n >= kBStages && !wait_chunk(c, kBarDone, kDoneStages, n - kBStages)) ok = false;
      ok = __all_sync(0xffffffffu, ok);
      if (reload && j == kChunks) {
        // the second half of the right operand: every slicer is past chunk 7
        slicer_sync();
        if (ok) {
          cp_async_block(c.sY, kLdY, reload, kK, ts, kStride);
          cp_async_wait_all();
        }
        slicer_sync();
      }
      if (ok) {
        uint8_t* stage = c.sB + (n % kBStages) * kBChunkBytes;
        for (; g < (j + 1) * 256; g += kStride) slice_b_quad<G>(c, stage, g & 255, (j % kChunks) * kKC);
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) mbar_arrive(c.bar + kBarBFull + n % kBStages);
      }
    }
  }
  // every thread: the last chunk's MMAs (and with them all earlier ones) are done
  if (ok && !wait_chunk(c, kBarDone, kDoneStages, n0 + nch - 1)) ok = false;
  tc_fence_after();
  c.n = n0 + nch;
  ok = __syncthreads_and(ok) != 0;   // uniform across the CTA
  if (!ok && threadIdx.x == 0) set_err(c);
  return ok;
}

// One output of a product from the words of its 8 t-group accumulators
// (column i of acc: FP32 images of exact integers g_t, |g_t| <= t 2^21, g_0 <=
// 2^19): V = sum_t g_t 2^(8 (7 - t)), |V| < 2^77, and the result V 2^k as
// binary64, rounded once to nearest even.  Results below 2^-1022 flush to
// zero, results of 2^1024 and above saturate to +-inf; valid == false gives 0.
//  * g_0..g_2 (|g| <= 2^22) come from the FP32 adder: the encoding of
//    g + 1.5 2^23 is g plus a constant (removed once, in the sum); the others
//    from the conversion unit.
//  * V = hi 2^32 + lo (64-bit Horner chains over t < 4 and t >= 4), then
//    V = vh 2^32 + vl with vl the low 32 bits of lo.
//  * X = V / 2^s rounded to odd (truncated, last bit set when a discarded bit
//    is), s the smallest shift that leaves |X| <= 2^62: when s > 0, X keeps 62
//    significant bits, so rounding X to 53 bits is the correct rounding of V
//    (rounding to odd at >= 55 bits makes the second rounding innocuous).
//  * |X| normalised, rounded to 53 bits and placed in the IEEE 754 encoding
//    with integer operations: on this part the FP64 pipe (which also converts
//    integers to binary64) is scarce, and the epilogue keeps it for the one
//    addition per element.
constexpr float kMagic = 12582912.0f;                                 // 1.5 2^23
constexpr long long kMagicSum = 0x4B400000LL * (16777216LL + 65536LL + 256LL);
__device__ __forceinline__ double recombine(const uint32_t (&acc)[kGroups][kDC], int i, int k,
                                            bool valid) {
  const long long b0 = __float_as_int(__uint_as_float(acc[0][i]) + kMagic);
  const long long b1 = __float_as_int(__uint_as_float(acc[1][i]) + kMagic);
  const long long b2 = __float_as_int(__uint_as_float(acc[2][i]) + kMagic);
  const long long g3 = __float2int_rn(__uint_as_float(acc[3][i]));
  const long long g4 = __float2int_rn(__uint_as_float(acc[4][i]));
  const long long g5 = __float2int_rn(__uint_as_float(acc[5][i]));
  const long long g6 = __float2int_rn(__uint_as_float(acc[6][i]));
  const long long g7 = __float2int_rn(__uint_as_float(acc[7][i]));
  const long long hi = b0 * 16777216LL + b1 * 65536LL + b2 * 256LL + (g3 - kMagicSum);
  const long long lo = g4 * 16777216LL + g5 * 65536LL + g6 * 256LL + g7;
  const long long vh = hi + (lo >> 32);                  // |vh| < 2^45
  const uint32_t vl = (uint32_t)lo;
  // s = bit length of |vh| (one's complement for negatives) beyond 30 bits, in [0, 15]
  const uint32_t top = (uint32_t)((unsigned long long)(vh ^ (vh >> 63)) >> 30);
  const int s = 32 - __clz((int)top);
  const uint32_t sticky = (uint32_t)((unsigned long long)vl << (32 - s)) != 0u ? 1u : 0u;
  const long long X =
      (long long)(((unsigned long long)vh << (32 - s)) | (unsigned long long)((vl >> s) | sticky));
  const unsigned long long sg = (unsigned long long)(X >> 63);
  const unsigned long long ax = ((unsigned long long)X ^ sg) - sg;   // |X| <= 2^62
  const int lz = __clzll((long long)ax);                 // 64 when X == 0
  const unsigned long long u = ax << (lz & 63);          // leading one at bit 63
  const unsigned long long m = u >> 11;                  // 53 significant bits
  const uint32_t low = (uint32_t)u & 0x7FFu;             // round half to even on the 11 dropped bits
  const unsigned long long mr = m + (((low + ((uint32_t)m & 1u)) > 0x400u) ? 1ULL : 0ULL);
  const int e = k + s + 1023 + 63 - lz;                  // biased exponent before a rounding carry
  // m carries its leading one into the exponent field (a rounding carry to
  // 2^53 bumps the exponent once more, with a zero fraction)
  const unsigned long long bits = mr + ((unsigned long long)(e - 1) << 52);
  const unsigned long long res =
      (!valid || ax == 0ULL || e < 1) ? 0ULL : (e > 2046 ? 0x7FF0000000000000ULL : bits);
  return __longlong_as_double((long long)(res | (sg & 0x8000000000000000ULL)));
}

// Epilogue modes (R = the product just computed).
enum Epi : int {
  kEpiStore = 0,      // g = R                                   (global)
  kEpiToY = 1,        // sY = gm + R (gm global, may be null)    -> next right operand
  kEpiToYSubTop = 2,  // sY = R; gm -= R (gm global, may be null) -> next right operand
  kEpiSubInto = 3,    // g -= R                                  (global)
};

// Recombine the 8 t-group accumulators into FP64 and apply the epilogue.
// Warp w handles TMEM lanes (rows) 32*(w%4).. and kColsPerWarp columns from
// kColsPerWarp*(w/4).  Ea: row exponents of X (global).  G = 4: groups 4..7
// are taken as zero.
template <int G = kGroups>
inline __device__ void drain(Ctx& c, const int* Ea, int mode, double* g, int ldg, double* gm,
                             int ldm) {
  static_assert(G == 8 || G == 4, "epilogue loads");
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int kColsPerWarp = kN / (kWarps / 4);
  static_assert(kColsPerWarp % kDC == 0, "epilogue passes");
  const int row = 32 * (w & 3) + lane;
  const int cb = kColsPerWarp * (w >> 2);
  const int ea = __ldcg(Ea + row);
  const uint32_t lane_addr = c.tmem + ((uint32_t)(32 * (w & 3)) << 16);
  const bool to_y = (mode == kEpiToY || mode == kEpiToYSubTop);
  const int nb = c.yb ^ 1;   // exponents of the new right operand
  if (to_y) {
    if (threadIdx.x < kN) c.sEb[nb * kN + threadIdx.x] = 0;
    __syncthreads();
  }
  // the memory operand of each mode
  const double* msrc = (mode == kEpiSubInto) ? g : (mode == kEpiStore) ? nullptr : gm;
  const int mld = (mode == kEpiSubInto) ? ldg : ldm;
#pragma unroll 1
  for (int pass = 0; pass < kColsPerWarp / kDC; pass++) {
    const int c0 = cb + kDC * pass;
    // issue the memory loads before the TMEM reads so they overlap
    double mem[kDC];
#pragma unroll
    for (int i = 0; i < kDC; i++) mem[i] = msrc ? ldg_cg(msrc + row + (size_t)(c0 + i) * mld) : 0.0;
    uint32_t acc[kGroups][kDC];
    if (G == 8)
      tmem_ld_groups(lane_addr + (uint32_t)c0, acc);
    else
      tmem_ld_groups4(lane_addr + (uint32_t)c0, acc);
#pragma unroll
    for (int i = 0; i < kDC; i++) {
      const int col = c0 + i;
      const int eb = c.sEb[c.yb * kN + col];
      const double r = recombine(acc, i, ea + eb - (kExpBias + 1023), ea > 0 && eb > 0);
      const size_t o = (size_t)col;
      double y = 0.0;
      if (mode == kEpiStore) {
        stg_cg(g + row + o * ldg, r);
      } else if (mode == kEpiToY) {
        y = mem[i] + r;
      } else if (mode == kEpiToYSubTop) {
        y = r;
        if (gm) stg_cg(gm + row + o * ldm, mem[i] - r);
      } else {
        stg_cg(g + row + o * ldg, mem[i] - r);
      }
      if (to_y) {
        c.sY[col * kLdY + row] = y;
        const unsigned e = __reduce_max_sync(0xffffffffu, (unsigned)biased_exp(y));
        if (lane == 0) atomicMax(c.sEb + nb * kN + col, (int)e);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (to_y) c.yb = nb;
}

// One product: X (prepared, row exponents Ea) times the staged right operand;
// Xnext: the next product's left operand (prefetched) or nullptr.  G: the
// t-groups kept (8: every product of weight <= 7, FP64-level; 4: weight <= 3,
// about 2^-30 of rowmax * colmax * K).
template <int G = kGroups>
inline __device__ bool product(Ctx& c, const uint8_t* Xprep, const uint8_t* Xnext, const int* Ea,
                               int mode, double* g, int ldg, double* gm, int ldm, int nch = kChunks,
                               const double* reload = nullptr) {
  if (!gemm<G>(c, Xprep, Xnext, nch, reload)) return false;
  drain<G>(c, Ea, mode, g, ldg, gm, ldm);
  return true;
}

// ---------------------------------------------------------------------------
// Preparation of a left operand (once per panel tile)
// ---------------------------------------------------------------------------
// Columns k < kcount of X(r, k) = acc(r, k) (kcount a multiple of kKC) into
// dst in the [kc][slice][core layout] order, with the row exponents sE
// (shared) already known.
template <class Acc>
inline __device__ void slice_cols(const Acc& acc, uint8_t* dst, const int* sE, int kcount) {
  const int quads = kK * kcount / 4;
  for (int qd = threadIdx.x; qd < quads; qd += kThreads) {
    const int r = qd % kK;
    const int k4 = (qd / kK) * 4;
    const int E = sE[r];
    float d[4][kS];
#pragma unroll
    for (int i = 0; i < 4; i++) digits(fixed_of(acc(r, k4 + i), E), d[i]);
    uint8_t* blk = dst + (size_t)(k4 / kKC) * kAChunkBytes;
    const int off = core_off(r, k4 % kKC);
#pragma unroll
    for (int p = 0; p < kS; p++) {
      uint2 w;
      w.x = bf16x2(d[0][p], d[1][p]);
      w.y = bf16x2(d[2][p], d[3][p]);
      *reinterpret_cast<uint2*>(blk + p * kSliceABytes + off) = w;
    }
  }
  fence_proxy_async_global();
  __syncthreads();
}

// Slice the 128 x 128 left operand X(r, k) = acc(r, k) into the
// [kc][slice][core layout] order at dst (global) and write its row exponents
// to Ea (global); sE: 128 ints of shared scratch.
template <class Acc>
inline __device__ void slice_left(const Acc& acc, uint8_t* dst, int* Ea, int* sE) {
  if (threadIdx.x < kK) {
    const int r = threadIdx.x;
    int e = 0;
#pragma unroll 8
    for (int k = 0; k < kK; k++) e = max(e, biased_exp(acc(r, k)));
    sE[r] = e;
    Ea[r] = e;
  }
  __syncthreads();
  slice_cols(acc, dst, sE, kK);
}

// A 128 x 128 column-major matrix in global memory (ld kK) as a left operand.
struct GlobalAcc {
  const double* g;
  __device__ __forceinline__ double operator()(int r, int k) const { return __ldcg(g + r + (size_t)k * kK); }
};

// Accessor of a 128 x 128 column-major matrix S staged in shared memory with
// leading dimension kLdT: X = S or X = S^T, with an element mask.
struct StagedAcc {
  const double* s;
  int rs, ks;   // X(r, k) = s[r * rs + k * ks]
  int kind;
  __device__ __forceinline__ double operator()(int r, int k) const {
    const double x = s[r * rs + k * ks];
    if (kind == kUnitLower) return (r > k) ? x : (r == k ? 1.0 : 0.0);
    if (kind == kUnitUpper) return (k > r) ? x : (k == r ? 1.0 : 0.0);
    if (kind == kUpperIncl) return (r <= k) ? x : 0.0;
    if (kind == kLowerIncl) return (r >= k) ? x : 0.0;
    return x;
  }
};

// Stage a 128 x 128 column-major tile (global, ld kK) in shared memory, ld kLdT.
__device__ __forceinline__ void stage_tile(double* s, const double* src) {
  constexpr int kIter = kK * kK / 2 / kThreads;   // pairs per thread
#pragma unroll 4
  for (int it = 0; it < kIter; it++) {
    const int e = threadIdx.x + it * kThreads;
    const int col = e / (kK / 2), r = 2 * (e % (kK / 2));
    const double2 v = __ldcg(reinterpret_cast<const double2*>(src + (size_t)col * kK + r));
    s[col * kLdT + r] = v.x;
    s[col * kLdT + r + 1] = v.y;
  }
  __syncthreads();
}

}  // namespace oz
}  // namespace hqr
