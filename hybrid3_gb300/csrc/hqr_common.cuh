// hqr_common.cuh -- shared device helpers for the GB300 tiled-QR kernels.
//
// Tile layout (the reference's, mat_prod.h:57-67): tile (i,j) of an MT x NT
// grid of NB x NB tiles starts at (i + j*MT)*NB*NB and is column-major with
// leading dimension NB; the TAU block of tile (i,j) starts at (i + j*MT)*NB.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace hqr {

constexpr int kThreads = 256;          // threads per CTA of every tile kernel
constexpr int kWarps = kThreads / 32;
constexpr int kMaxNB = 512;
constexpr int kMaxIB = 64;

// Error word bits written by device code (never a trap): the host turns them
// into a status code.
enum DevErr : int {
  kErrNone = 0,
  kErrTimeout = 1,        // a bounded wait ran out
  kErrBadTask = 2,        // a queue slot held an invalid task id
  kErrBadShape = 4,       // kernel launched with an unsupported NB/IB
};

// L2-only global accesses.  Tiles are rewritten by other CTAs while this one
// may still hold a line in its SM's (non-coherent) L1, so every tile access
// bypasses L1.
__device__ __forceinline__ double ldg_cg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ void stg_cg(double* p, double v) { __stcg(p, v); }

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of one double per thread; red must hold kWarps doubles.
// Every thread gets the result.
__device__ __forceinline__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < kWarps; i++) s += red[i];
  return s;
}

__device__ __forceinline__ size_t tile_off(int i, int j, int MT, int NB) {
  return ((size_t)i + (size_t)j * MT) * (size_t)NB * NB;
}
__device__ __forceinline__ size_t tau_off(int i, int j, int MT, int NB) {
  return ((size_t)i + (size_t)j * MT) * (size_t)NB;
}

}  // namespace hqr
