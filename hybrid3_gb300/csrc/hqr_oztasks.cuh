// hqr_oztasks.cuh -- tile tasks of the split-precision path.
//
//   OZPREP(i,k): full NB x NB upper T of panel tile (k,i) (LAPACK dlarft,
//     forward, columnwise, from V and TAU -- the rebuild Hybrid_make_Q does
//     with IB = NB, Hybrid_make_Q.c:124-130,159-163) and the sliced left
//     operands V^T, T^T and V of that tile.
//   OZAPPLY: one 64-column block of a LARFB (CORE_dormqr, V unit lower) or
//     SSRFB (CORE_dtsmqr, V dense) as three Ozaki products on the tensor
//     cores:  W = C_top + V^T C_bot;  W2 = T^T W;  C_top -= W2;  C_bot -= V W2.
#pragma once
#include "hqr_ozaki.cuh"

namespace hqr {

// dlarft 'F','C' with k = NB: T (global, NB x NB, ld NB) from V (global) and
// TAU.  unit: V is the unit-lower part of a GEQRT tile, else a dense TS V
// (whose top part is the identity).  g: NB doubles of shared memory.
inline __device__ void build_full_t(const double* V, const double* tau, double* T, bool unit, int NB,
                                    double* g) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int c = 0; c < NB; c++) {
    const double* vc = V + (size_t)c * NB;
    for (int a = warp; a < c; a += kWarps) {
      const double* va = V + (size_t)a * NB;
      double s = 0.0;
      for (int r = (unit ? c + 1 : 0) + lane; r < NB; r += 32) s = fma(ldg_cg(va + r), ldg_cg(vc + r), s);
      s = warp_sum(s);
      if (lane == 0) g[a] = unit ? s + ldg_cg(va + c) : s;
    }
    __syncthreads();
    const double tc = ldg_cg(tau + c);
    for (int a = threadIdx.x; a < NB; a += kThreads) {
      double v;
      if (a < c) {
        double s = 0.0;
        for (int b = a; b < c; b++) s = fma(ldg_cg(T + a + (size_t)b * NB), g[b], s);
        v = (tc == 0.0) ? 0.0 : -tc * s;
      } else {
        v = (a == c) ? tc : 0.0;
      }
      stg_cg(T + a + (size_t)c * NB, v);
    }
    __syncthreads();
  }
}

// Slice-store layout of a panel tile: [V^T | T^T | V], each oz::operand_bytes(NB).
template <class SC>
__device__ void prep_operands(const double* V, const double* T, bool unit, int NB, uint8_t* slices,
                              int* exps) {
  const size_t ob = oz::operand_bytes(NB);
  oz::prep_operand<SC>(V, NB, 1, NB, slices, exps, unit ? 2 : 0);                 // V^T
  oz::prep_operand<SC>(T, NB, 1, NB, slices + ob, exps + NB, 3);                  // T^T
  oz::prep_operand<SC>(V, 1, NB, NB, slices + 2 * ob, exps + 2 * NB, unit ? 1 : 0);  // V
}
inline __device__ void task_ozprep(const double* V, const double* tau, double* T, bool unit, int NB,
                                   uint8_t* slices, int* exps, double* smem) {
  build_full_t(V, tau, T, unit, NB, smem);
  if (NB <= 128)
    prep_operands<oz::Scheme8x7>(V, T, unit, NB, slices, exps);
  else
    prep_operands<oz::Scheme7x8>(V, T, unit, NB, slices, exps);
}

// One 64-column block of the update.  Ctop: A1 block (SSRFB) or nullptr
// (LARFB); Cbot: A2 block (SSRFB) or the C block (LARFB); ld NB.  W, W2:
// per-CTA scratch of NB x 64 doubles (ld NB).  Returns false on a device
// time-out (error word already set).
template <class SC>
__device__ bool ozapply_products(oz::Ctx& c, int NB, const uint8_t* slices, const int* exps, bool unit,
                                 double* Ctop, double* Cbot, double* W, double* W2) {
  const size_t ob = oz::operand_bytes(NB);
  if (!oz::product<SC>(c, NB, slices, exps, unit ? 2 : 0, Cbot, NB, oz::kEpiStoreAdd, W, NB, Ctop,
                       NB, nullptr, 0))
    return false;
  if (!oz::product<SC>(c, NB, slices + ob, exps + NB, 1, W, NB, oz::kEpiStoreSub, W2, NB, nullptr,
                       0, Ctop, NB))
    return false;
  return oz::product<SC>(c, NB, slices + 2 * ob, exps + 2 * NB, unit ? 1 : 0, W2, NB,
                         oz::kEpiSubInto, Cbot, NB, nullptr, 0, nullptr, 0);
}
inline __device__ bool task_ozapply(oz::Ctx& c, int NB, const uint8_t* slices, const int* exps,
                                    bool unit, double* Ctop, double* Cbot, double* W, double* W2) {
  const bool ok = (NB <= 128)
                      ? ozapply_products<oz::Scheme8x7>(c, NB, slices, exps, unit, Ctop, Cbot, W, W2)
                      : ozapply_products<oz::Scheme7x8>(c, NB, slices, exps, unit, Ctop, Cbot, W, W2);
  if (!ok) return false;
  // every copy and MMA has completed: release the barriers, whose shared
  // memory the next task may use for other data
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 0; i < 4; i++)
      asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(oz::smem_u32(c.bar + i)) : "memory");
  __syncthreads();
  return true;
}

}  // namespace hqr
