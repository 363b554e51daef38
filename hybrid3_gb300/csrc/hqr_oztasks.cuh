// hqr_oztasks.cuh -- tile tasks of the split-precision path (NB = 128).
//
//   OZPREP(i,k): the sliced left operands V^T, T^T and V of panel tile (k,i),
//     with the full NB x NB upper T of the tile (LAPACK dlarft, forward,
//     columnwise, from V and TAU -- the rebuild Hybrid_make_Q does with
//     IB = NB, Hybrid_make_Q.c:124-130,159-163).  G = V^T V runs on the tensor
//     cores (two products); the T recurrence runs in shared memory.
//   OZAPPLY: one 64-column block of a LARFB (CORE_dormqr, V unit lower) or
//     SSRFB (CORE_dtsmqr, V dense) as three products:
//       W = C_top + V^T C_bot;  W2 = T^T W;  C_top -= W2;  C_bot -= V W2,
//     with W and W2 kept in shared memory between the products.
#pragma once
#include "hqr_ozaki.cuh"

namespace hqr {

// Slots of a panel tile's prepared operands (and of their row exponents):
// V^T, the middle operand (T^T, or T where the preparation applies H itself),
// V, and -- written by the factorization's preparation only -- T, so that Q
// generation (which applies H, not H^T) can reuse the factorization's slices.
constexpr size_t kOzVT = 0, kOzTT = 1, kOzV = 2, kOzT = 3;

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

// OZPREP of panel tile V (global, NB x NB, of shape vkind) with TAU tau.  G: NB x NB global scratch.
// slices / exps: this tile's prepared operands and row exponents; the middle
// operand is T^T (applying H^T) or, with t_transposed false, T (applying H);
// with also_t, T goes to slot kOzT as well.  sm: the CTA's dynamic shared
// memory (oz::kSmemBytes).  False on a device time-out.
inline __device__ bool task_ozprep(const double* V, const double* tau, double* G, int vkind,
                                   uint8_t* slices, int* exps, uint8_t* sm, uint32_t tmem,
                                   unsigned* err, bool t_transposed, bool also_t) {
  using namespace oz;
  constexpr size_t ob = operand_bytes();
  // 1. V^T and V from a shared-memory copy of the tile
  {
    double* sV = reinterpret_cast<double*>(sm);
    int* sE = reinterpret_cast<int*>(sm + kLdT * kK * 8);
    stage_tile(sV, V);
    const int kt = vkind == kVUnitLower ? kUnitUpper : vkind == kVUpper ? kLowerIncl : kDense;
    const int kv = vkind == kVUnitLower ? kUnitLower : vkind == kVUpper ? kUpperIncl : kDense;
    slice_left(StagedAcc{sV, kLdT, 1, kt}, slices + kOzVT * ob, exps + kOzVT * kK, sE);
    slice_left(StagedAcc{sV, 1, kLdT, kv}, slices + kOzV * ob, exps + kOzV * kK, sE);
  }
  // 2. G = V^T V on the tensor cores, by 64-column blocks, into G (global)
  {
    Ctx c;
    ctx_init(c, sm, tmem, err);
    for (int cb = 0; cb < kK / kN; cb++) {
      prefetch(c, slices + kOzVT * ob);
      stage_y(c, V + (size_t)cb * kN * kK, kK, vkind == kVDense ? -1 : cb * kN, vkind == kVUpper);
      if (!product(c, slices + kOzVT * ob, (cb + 1 < kK / kN) ? slices + kOzVT * ob : nullptr,
                   exps + kOzVT * kK, kEpiStore, G + (size_t)cb * kN * kK, kK, nullptr, 0))
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
  // 4. T^T or T (and T)
  slice_left(PackedTAcc{sT, t_transposed}, slices + kOzTT * ob, exps + kOzTT * kK, sE);
  if (also_t) slice_left(PackedTAcc{sT, false}, slices + kOzT * ob, exps + kOzT * kK, sE);
  return true;
}

// One 64-column block of the update.  Ctop: A1 block (SSRFB) or nullptr
// (LARFB); Cbot: A2 block (SSRFB) or the C block (LARFB); ld NB.  mid: the
// slot of the middle operand (kOzTT, or kOzT for Q generation on the
// factorization's slices).  Returns false on a device time-out (error word
// already set).  G: t-groups of the three products (8: FP64-level; 4: the
// reduced form, see oz::product).
template <int G = oz::kGroups>
inline __device__ bool task_ozapply(oz::Ctx& c, const uint8_t* slices, const int* exps, double* Ctop,
                                    double* Cbot, int mid) {
  using namespace oz;
  constexpr size_t ob = operand_bytes();
  prefetch<G>(c, slices + kOzVT * ob);
  stage_y(c, Cbot, kK, -1);
  if (!product<G>(c, slices + kOzVT * ob, slices + mid * ob, exps + kOzVT * kK, kEpiToY, nullptr, 0, Ctop, kK))
    return false;
  if (!product<G>(c, slices + mid * ob, slices + kOzV * ob, exps + mid * kK, kEpiToYSubTop, nullptr, 0, Ctop,
                  kK))
    return false;
  if (!product<G>(c, slices + kOzV * ob, nullptr, exps + kOzV * kK, kEpiSubInto, Cbot, kK, nullptr, 0))
    return false;
  ctx_release(c);
  return true;
}

}  // namespace hqr
