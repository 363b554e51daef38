// hqr_oztest.cu -- the split-precision product engine on its own: C = X Y for
// a 128 x 128 left operand X and a 128 x 64 right operand Y (column-major
// FP64), through exactly the slicing, tcgen05 products and recombination the
// update tasks use.  A diagnostic / unit-test entry point.
#include "hqr_ozaki.cuh"
#include "hqr_internal.h"

namespace hqr {

__global__ void __launch_bounds__(kThreads, 1) k_ozaki_product(const double* X, const double* Y, double* C,
                                                             uint8_t* prep, int* exps, unsigned* err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  __shared__ uint32_t s_tmem;
  if ((threadIdx.x >> 5) == 0) oz::tmem_alloc(&s_tmem, 512);
  oz::tc_fence_before();
  __syncthreads();
  oz::tc_fence_after();
  {
    double* sX = reinterpret_cast<double*>(sm);
    int* sE = reinterpret_cast<int*>(sm + oz::kLdT * oz::kK * 8);
    oz::stage_tile(sX, X);
    oz::slice_left(oz::StagedAcc{sX, 1, oz::kLdT, oz::kDense}, prep, exps, sE);
  }
  oz::Ctx c;
  oz::ctx_init(c, sm, s_tmem, err);
  oz::prefetch(c, prep);
  oz::stage_y(c, Y, oz::kK, -1);
  if (oz::product(c, prep, nullptr, exps, oz::kEpiStore, C, oz::kK, nullptr, 0)) oz::ctx_release(c);
  oz::tc_fence_before();
  __syncthreads();
  oz::tc_fence_after();
  if ((threadIdx.x >> 5) == 0) oz::tmem_dealloc(s_tmem, 512);
}

}  // namespace hqr

extern "C" int hqr_ozaki_product(int NB, const double* dX, const double* dY, double* dC, void* stream) {
  if (!dX || !dY || !dC) return HQR_ERR_INVALID;
  if (NB != hqr::oz::kK) return HQR_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  uint8_t* prep = nullptr;
  int* exps = nullptr;
  unsigned* err = nullptr;
  if (cudaMalloc(&prep, hqr::oz::operand_bytes()) != cudaSuccess ||
      cudaMalloc(&exps, NB * sizeof(int)) != cudaSuccess || cudaMalloc(&err, sizeof(unsigned)) != cudaSuccess) {
    cudaFree(prep);
    cudaFree(exps);
    return HQR_ERR_NOMEM;
  }
  cudaMemsetAsync(err, 0, sizeof(unsigned), s);
  cudaFuncSetAttribute(hqr::k_ozaki_product, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       hqr::oz::kSmemBytes);
  hqr::k_ozaki_product<<<1, hqr::kThreads, hqr::oz::kSmemBytes, s>>>(dX, dY, dC, prep, exps, err);
  unsigned herr = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(prep);
  cudaFree(exps);
  cudaFree(err);
  if (e != cudaSuccess) return hqr::record_cuda_error(e, "hqr_ozaki_product");
  return herr ? HQR_ERR_TIMEOUT : HQR_OK;
}
