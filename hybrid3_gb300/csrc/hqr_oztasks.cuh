// hqr_oztasks.cuh -- tile tasks of the split-precision path (NB = 128).
//
// A block reflector H = I - [I; V] T [I; V]^T applied as H^T (the
// factorization, Q^T C; CORE_dtsmqr / CORE_dormqr) or as H (Q generation)
// to a column block [C_top; C_bot] needs W2 = M (C_top + V^T C_bot), M = T^T
// or T, then C_top -= W2 and C_bot -= V W2.  With Z = M V^T prepared once per
// panel tile, W2 = Z C_bot + M C_top is ONE product of K = 256:
//
//   OZPREP(i,k): T from V and TAU (LAPACK dlarft, forward, columnwise -- the
//     full NB x NB T Hybrid_make_Q rebuilds with IB = NB,
//     Hybrid_make_Q.c:124-130,159-163; G = V^T V on the tensor cores, the
//     recurrence in shared memory), Z = M V^T on the tensor cores, and the
//     sliced left operands X1 = [Z | M] (128 x 256, one row exponent per row
//     over both halves) and V.
//   OZAPPLY: one 64-column block of an SSRFB (V dense) or LARFB (V unit
//     lower, no C_top) as two products:
//       W2 = [Z | M] [C_bot; C_top]   (LARFB: Z C)  -> C_top -= W2
//       C_bot -= V W2,
//     with W2 kept in shared memory between them: two epilogues per task.
#pragma once
#include "hqr_ozaki.cuh"

namespace hqr {

// Slots of a panel tile's prepared operands (operand_bytes() each) and of
// their row exponents (kK ints each): X1 = [Z | M] (slots 0-1: 16 K chunks,
// one exponent per row in slot 0), V (slot 2), and slot 3, scratch of the
// preparation (V^T, then M with its own exponents).
constexpr size_t kOzX = 0, kOzV = 2, kOzS = 3;

// T upper triangular, packed by columns in shared memory: T(a, b) (a <= b)
// at b (b + 1) / 2 + a.  As a left operand: X = T^T (transposed) or X = T.
struct PackedTAcc {
  const double* t;
  bool transposed;
  __device__ __forceinline__ double operator()(int r, int k) const {
    if (transposed) return (k <= r) ? t[r * (r + 1) / 2 + k] : 0.0;   // T^T(r, k) = T(k, r)
    return (r <= k) ? t[k * (k + 1) / 2 + r] : 0.0;
  }
};

// T recurrence (dlarft 'F','C', k = NB = 128) in shared memory,
//   T(c, c) = tau_c;  T(0:c, c) = -tau_c T(0:c, 0:c) G(0:c, c)  (zero when tau_c = 0),
// regrouped by blocks of 16 columns: first the diagonal 16 x 16 blocks (each
// row runs its own scalar recurrence over its own row: no barrier), then for
// block columns b = 1..7
//   X = G(0:bw, bw:bw+16) T_bb,   T(0:bw, bw:bw+16) = -T(0:bw, 0:bw) X,
// the same sums (tau_c = 0 leaves column c zero either way).  FP64 on this
// part issues one warp instruction per ~19 cycles per SM, so the work is laid
// out for full warps: the triangular product pairs rows r and bw-1-r, whose
// dots add up to bw + 1 terms.  The scalar column recurrence left most lanes
// of a warp idle on the short rows and took 2.6x longer.
// sG: strictly upper part of G = V^T V, packed: G(b, c) (b < c) at c (c - 1) / 2 + b.
// sT: the result, packed upper: T(a, b) (a <= b) at b (b + 1) / 2 + a.
// sX: (NB - 16) x 16 doubles of scratch.
inline __device__ void t_recurrence(const double* sG, double* sT, double* sX, const double* tau) {
  constexpr int K = oz::kK, BS = 16;
  const int tid = threadIdx.x;
  if (tid < K) {
    const int b = tid / BS, a = tid % BS;
    for (int c = a; c < BS; c++) {
      const int gc = b * BS + c;
      const double tc = __ldcg(tau + gc);
      double s = 0.0;
      for (int d = a; d < c; d++) {
        const int gd = b * BS + d;
        s = fma(sT[gd * (gd + 1) / 2 + tid], sG[gc * (gc - 1) / 2 + gd], s);
      }
      sT[gc * (gc + 1) / 2 + tid] = (c == a) ? tc : (tc == 0.0 ? 0.0 : -tc * s);
    }
  }
  __syncthreads();
  for (int b = 1; b < K / BS; b++) {
    const int bw = b * BS;
    for (int e = tid; e < bw * BS; e += kThreads) {
      const int r = e % bw, j = e / bw;
      double s = 0.0;
      for (int d = 0; d <= j; d++)
        s = fma(sG[(bw + d) * (bw + d - 1) / 2 + r], sT[(bw + j) * (bw + j + 1) / 2 + bw + d], s);
      sX[r + j * bw] = s;
    }
    __syncthreads();
    for (int e = tid; e < (bw / 2) * BS; e += kThreads) {
      const int r0 = e % (bw / 2), j = e / (bw / 2), r1 = bw - 1 - r0;
      double s0 = 0.0, s1 = 0.0;
      for (int d = r0; d < bw; d++) s0 = fma(sT[d * (d + 1) / 2 + r0], sX[d + j * bw], s0);
      for (int d = r1; d < bw; d++) s1 = fma(sT[d * (d + 1) / 2 + r1], sX[d + j * bw], s1);
      const int cj = bw + j;
      sT[cj * (cj + 1) / 2 + r0] = -s0;
      sT[cj * (cj + 1) / 2 + r1] = -s1;
    }
    __syncthreads();
  }
}

// Shape of a panel tile's reflectors V.
enum VKind : int {
  kVDense = 0,       // TSQRT: the whole tile
  kVUnitLower = 1,   // GEQRT: strictly below the diagonal, unit diagonal
  kVUpper = 2,       // TT merge: the upper triangle with the diagonal
};

// OZPREP of panel tile V (global, NB x NB, of shape vkind) with TAU tau.
// G: NB x NB global scratch (it ends holding M).  slices / exps: this tile's
// prepared operands and row exponents; M = T^T (applying H^T) or, with
// t_transposed false, T (applying H).  sm: the CTA's dynamic shared memory
// (oz::kSmemBytes).  False on a device time-out.
inline __device__ bool task_ozprep(const double* V, const double* tau, double* G, int vkind,
                                   uint8_t* slices, int* exps, uint8_t* sm, uint32_t tmem,
                                   unsigned* err, bool t_transposed) {
  using namespace oz;
  constexpr size_t ob = operand_bytes();
  uint8_t* X1 = slices + kOzX * ob;
  uint8_t* XV = slices + kOzV * ob;
  uint8_t* XS = slices + kOzS * ob;
  // Z (FP64, ld kK) waits in X1's last 4 chunks until X1 is sliced
  double* Zs = reinterpret_cast<double*>(X1 + 12 * (size_t)kAChunkBytes);
  static_assert(12 * kAChunkBytes + kK * kK * 8 == 2 * operand_bytes(), "Z scratch");
  const int kv = vkind == kVUnitLower ? kUnitLower : vkind == kVUpper ? kUpperIncl : kDense;
  // 1. V^T (scratch) and V from a shared-memory copy of the tile
  {
    double* sV = reinterpret_cast<double*>(sm);
    int* sE = reinterpret_cast<int*>(sm + kLdT * kK * 8);
    stage_tile(sV, V);
    const int kt = vkind == kVUnitLower ? kUnitUpper : vkind == kVUpper ? kLowerIncl : kDense;
    slice_left(StagedAcc{sV, kLdT, 1, kt}, XS, exps + kOzS * kK, sE);
    slice_left(StagedAcc{sV, 1, kLdT, kv}, XV, exps + kOzV * kK, sE);
  }
  // 2. G = V^T V on the tensor cores, by 64-column blocks, into G (global)
  {
    Ctx c;
    ctx_init(c, sm, tmem, err);
    for (int cb = 0; cb < kK / kN; cb++) {
      prefetch(c, XS);
      stage_y(c, V + (size_t)cb * kN * kK, kK, vkind == kVDense ? -1 : cb * kN, vkind == kVUpper);
      if (!product(c, XS, (cb + 1 < kK / kN) ? XS : nullptr, exps + kOzS * kK, kEpiStore,
                   G + (size_t)cb * kN * kK, kK, nullptr, 0))
        return false;
    }
    ctx_release(c);
  }
  __threadfence_block();
  // 3. T in shared memory
  double* sG = reinterpret_cast<double*>(sm);
  double* sT = sG + kK * (kK - 1) / 2;
  int* sE = reinterpret_cast<int*>(sT + kK * (kK + 1) / 2);
  double* sX = reinterpret_cast<double*>(sE + kK);
  static_assert((kK * (kK - 1) / 2 + kK * (kK + 1) / 2) * 8 + kK * 4 + (kK - 16) * 16 * 8 <= kSmemBytes,
                "T recurrence scratch");
  constexpr int kPacked = kK * (kK - 1) / 2;
#pragma unroll 4
  for (int idx = threadIdx.x; idx < kPacked; idx += kThreads) {
    // column c of packed index idx: c (c - 1) / 2 <= idx < (c + 1) c / 2
    int c = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)idx)) * 0.5f);
    while (c * (c - 1) / 2 > idx) c--;
    while ((c + 1) * c / 2 <= idx) c++;
    sG[idx] = __ldcg(G + (idx - c * (c - 1) / 2) + (size_t)c * kK);
  }
  __syncthreads();
  t_recurrence(sG, sT, sX, tau);
  // 4. M to G (global, its last use of G was above) and sliced with its own
  //    row exponents into the scratch slot (V^T is not needed any more)
  {
    const PackedTAcc m{sT, t_transposed};
    for (int e = threadIdx.x; e < kK * kK; e += kThreads) stg_cg(G + e, m(e % kK, e / kK));
    slice_left(m, XS, exps + kOzS * kK, sE);
  }
  // 5. Z = M V^T on the tensor cores, into Zs
  {
    Ctx c;
    ctx_init(c, sm, tmem, err);
    for (int cb = 0; cb < kK / kN; cb++) {
      prefetch(c, XS);
      stage_yt(c, V, cb * kN, kv);
      if (!product(c, XS, (cb + 1 < kK / kN) ? XS : nullptr, exps + kOzS * kK, kEpiStore,
                   Zs + (size_t)cb * kN * kK, kK, nullptr, 0))
        return false;
    }
    ctx_release(c);
  }
  __threadfence_block();
  // 6. row exponents of X1 = [Z | M] over both halves
  //    (threads 0..127 scan Z's rows, threads 128..255 M's)
  static_assert(kThreads == 2 * kK, "one thread per row and half");
  int* sE1 = reinterpret_cast<int*>(sm);
  if (threadIdx.x < kK) sE1[threadIdx.x] = 0;
  __syncthreads();
  {
    const int r = threadIdx.x % kK;
    const double* src = threadIdx.x < kK ? Zs : G;
    int e = 0;
#pragma unroll 8
    for (int k = 0; k < kK; k++) e = max(e, biased_exp(__ldcg(src + r + (size_t)k * kK)));
    atomicMax(sE1 + r, e);
  }
  __syncthreads();
  if (threadIdx.x < kK) exps[kOzX * kK + threadIdx.x] = sE1[threadIdx.x];
  // 7. X1: Z into chunks 0-7 (all of Zs read before chunks 12-15 are written),
  //    then M into chunks 8-15
  slice_cols(GlobalAcc{Zs}, X1, sE1, kK);
  slice_cols(GlobalAcc{G}, X1 + (size_t)kChunks * kAChunkBytes, sE1, kK);
  return true;
}

// One 64-column block of the update.  Ctop: A1 block (SSRFB) or nullptr
// (LARFB); Cbot: A2 block (SSRFB) or the C block (LARFB); ld NB.  Returns
// false on a device time-out (error word already set).  G: t-groups of the
// products (8: FP64-level; 4: the reduced form, see oz::product).
template <int G = oz::kGroups>
inline __device__ bool task_ozapply(oz::Ctx& c, const uint8_t* slices, const int* exps, double* Ctop,
                                    double* Cbot) {
  using namespace oz;
  constexpr size_t ob = operand_bytes();
  const uint8_t* X1 = slices + kOzX * ob;
  const uint8_t* XV = slices + kOzV * ob;
  prefetch<G>(c, X1);
  // the right operand [C_bot; C_top]: C_bot staged, C_top loaded after chunk 7;
  // column exponents over both
  stage_y(c, Cbot, kK, -1, false, Ctop);
  if (!product<G>(c, X1, XV, exps + kOzX * kK, kEpiToYSubTop, nullptr, 0, Ctop, kK,
                  Ctop ? 2 * kChunks : kChunks, Ctop))
    return false;
  if (!product<G>(c, XV, nullptr, exps + kOzV * kK, kEpiSubInto, Cbot, kK, nullptr, 0)) return false;
  ctx_release(c);
  return true;
}

}  // namespace hqr
