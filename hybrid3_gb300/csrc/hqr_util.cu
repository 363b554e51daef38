// hqr_util.cu -- data-preparation and verification kernels around the QR path:
// the seeded uniform generator, identity / reflector-zeroing (Hybrid_make_I,
// the V zeroing of Hybrid_make_Q), the tile-wise C = A^T B of Hybrid_dgemm,
// Frobenius-norm reductions and the max column abs-sum of mat_comp3.
#include "hqr_common.cuh"
#include "hqr_internal.h"

namespace hqr {

// splitmix64 of (seed, column-major index) -> 53-bit uniform in [0,1) -> 2u-1.
__device__ __forceinline__ double uniform_pm1(uint64_t seed, uint64_t idx) {
  uint64_t z = idx + seed * 0x9E3779B97F4A7C15ull + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
  return 2.0 * u - 1.0;
}

// Element e of the tile array -> (row, column) of the matrix.
__device__ __forceinline__ void tile_rc(size_t e, int MT, int NB, long* r, long* c) {
  const size_t t2 = (size_t)NB * NB;
  const size_t tile = e / t2, in = e % t2;
  const int ti = (int)(tile % MT), tj = (int)(tile / MT);
  *r = (long)ti * NB + (long)(in % NB);
  *c = (long)tj * NB + (long)(in / NB);
}

__global__ void k_fill_uniform(double* A, long M, long N, int NB, uint64_t seed) {
  const int MT = (int)(M / NB);
  const size_t n = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    long r, c;
    tile_rc(e, MT, NB, &r, &c);
    A[e] = uniform_pm1(seed, (uint64_t)c * (uint64_t)M + (uint64_t)r);
  }
}

__global__ void k_identity(double* Q, long M, long N, int NB, int zero_first) {
  const int MT = (int)(M / NB);
  const size_t n = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    long r, c;
    tile_rc(e, MT, NB, &r, &c);
    if (r == c) Q[e] = 1.0;
    else if (zero_first) Q[e] = 0.0;
  }
}

// In-place transpose of a square tile-layout matrix, by 32 x 32 blocks (each
// inside one tile): the CTA of block (bi, bj), bi <= bj, swaps the transposes
// of blocks (bi, bj) and (bj, bi) through shared memory.  Block 32 x 8.
__global__ void k_transpose_tiles(double* Q, long N, int NB) {
  __shared__ double a[32][33], b[32][33];
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bi > bj) return;
  const int MT = (int)(N / NB);
  const int tx = threadIdx.x, ty = threadIdx.y;
  auto at = [&](long R, long C) -> size_t {
    return ((size_t)(R / NB) + (size_t)(C / NB) * MT) * (size_t)NB * NB + (size_t)(R % NB) +
           (size_t)(C % NB) * NB;
  };
  const long r0 = 32L * bi, c0 = 32L * bj;
  for (int y = ty; y < 32; y += 8) {
    a[y][tx] = Q[at(r0 + tx, c0 + y)];
    if (bi != bj) b[y][tx] = Q[at(c0 + tx, r0 + y)];
  }
  __syncthreads();
  for (int y = ty; y < 32; y += 8) {
    Q[at(c0 + tx, r0 + y)] = a[tx][y];
    if (bi != bj) Q[at(r0 + tx, c0 + y)] = b[tx][y];
  }
}

// Streaming copy of n doubles by SM loads and stores (one side may be a
// page-locked host array's device mapping); vec: both addresses 16-byte
// aligned.
__global__ void k_copy_stream(double* __restrict__ dst, const double* __restrict__ src, size_t n, int vec) {
  const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
  if (vec) {
    const size_t n2 = n / 2;
    for (size_t i = tid; i < n2; i += stride)
      reinterpret_cast<double2*>(dst)[i] = reinterpret_cast<const double2*>(src)[i];
    if (tid == 0 && (n & 1)) dst[n - 1] = src[n - 1];
  } else {
    for (size_t i = tid; i < n; i += stride) dst[i] = src[i];
  }
}

// Zero V: the strictly lower part of the diagonal tiles (i,i) and every tile
// (k,i), k > i, of the first min(MT, NT) tile columns.
__global__ void k_zero_reflectors(double* A, long M, long N, int NB) {
  const int MT = (int)(M / NB), NT = (int)(N / NB);
  const int steps = MT < NT ? MT : NT;
  const size_t n = (size_t)M * (size_t)steps * NB;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    long r, c;
    tile_rc(e, MT, NB, &r, &c);
    const long ti = r / NB, tj = c / NB;
    if (ti > tj || (ti == tj && r > c)) A[e] = 0.0;
  }
}

// C(i,j) = sum_k A(k,i)^T B(k,j) for tiles: one CTA per 64 x 64 output block.
constexpr int kGB = 64, kGK = 16;
__global__ void __launch_bounds__(256) k_dgemm_tn(const double* __restrict__ A, const double* __restrict__ B,
                                                  double* __restrict__ C, long M, long N, int NB) {
  const int MT = (int)(M / NB), NT = (int)(N / NB);
  const int bpt = NB / kGB > 0 ? NB / kGB : 1;          // 64-blocks per tile side
  const int nb_blk = (NB < kGB) ? NB : kGB;
  const int ti = blockIdx.y / bpt, bi = blockIdx.y % bpt;
  const int tj = blockIdx.x / bpt, bj = blockIdx.x % bpt;
  if (ti >= NT || tj >= NT) return;
  __shared__ double sA[kGK][kGB + 1];
  __shared__ double sB[kGK][kGB + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4] = {};
  for (int tk = 0; tk < MT; tk++) {
    const double* a = A + ((size_t)tk + (size_t)ti * MT) * NB * NB + (size_t)bi * nb_blk * NB;
    const double* b = B + ((size_t)tk + (size_t)tj * MT) * NB * NB + (size_t)bj * nb_blk * NB;
    for (int k0 = 0; k0 < NB; k0 += kGK) {
      __syncthreads();
      for (int e = threadIdx.x; e < kGK * kGB; e += 256) {
        const int kk = e % kGK, col = e / kGK;
        sA[kk][col] = (col < nb_blk) ? a[(size_t)col * NB + k0 + kk] : 0.0;
        sB[kk][col] = (col < nb_blk) ? b[(size_t)col * NB + k0 + kk] : 0.0;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < kGK; kk++) {
        double av[4], bv[4];
#pragma unroll
        for (int q = 0; q < 4; q++) { av[q] = sA[kk][ty + 16 * q]; bv[q] = sB[kk][tx + 16 * q]; }
#pragma unroll
        for (int p = 0; p < 4; p++)
#pragma unroll
          for (int q = 0; q < 4; q++) acc[p][q] = fma(av[p], bv[q], acc[p][q]);
      }
    }
  }
  double* c = C + ((size_t)ti + (size_t)tj * MT) * NB * NB + (size_t)bj * nb_blk * NB + (size_t)bi * nb_blk;
#pragma unroll
  for (int p = 0; p < 4; p++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int r = ty + 16 * p, col = tx + 16 * q;
      if (r < nb_blk && col < nb_blk) c[(size_t)col * NB + r] = acc[p][q];
    }
}

__global__ void k_frob_diff(const double* X, const double* Y, double alpha, long M, long N, int NB,
                            double* out) {
  const int MT = (int)(M / NB);
  const size_t n = (size_t)M * N;
  double s = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    double v = X[e];
    if (Y) v -= Y[e];
    if (alpha != 0.0) {
      long r, c;
      tile_rc(e, MT, NB, &r, &c);
      if (r == c) v -= alpha;
    }
    s = fma(v, v, s);
  }
  s = warp_sum(s);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) atomicAdd(out, v);
  }
}

__global__ void k_tiles_to_colmajor(const double* T, double* out, long M, long N, int NB, int to_cm) {
  const int MT = (int)(M / NB);
  const size_t n = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    long r, c;
    tile_rc(e, MT, NB, &r, &c);
    const size_t cm = (size_t)c * M + r;
    if (to_cm) out[cm] = T[e]; else out[e] = T[cm];
  }
}

// Padded conversions: the tile array holds an (MT NB) x (NT NB) matrix, MT =
// ceil(M / NB), NT = ceil(N / NB); the column-major matrix is M x N with
// leading dimension ld.  Into tiles the tail rows and columns are zero; out of
// tiles only the leading M x N block is written.  One thread per tile element.
__global__ void k_colmajor_to_tiles_padded(const double* __restrict__ in, long ld, long M, long N, int NB,
                                           int MT, int NT, double* __restrict__ T) {
  const size_t n = (size_t)MT * NT * NB * NB;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    long r, c;
    tile_rc(e, MT, NB, &r, &c);
    T[e] = (r < M && c < N) ? in[(size_t)c * ld + r] : 0.0;
  }
}
__global__ void k_tiles_to_colmajor_padded(const double* __restrict__ T, long ld, long M, long N, int NB,
                                           int MT, double* __restrict__ out) {
  const size_t n = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const long r = (long)(e % (size_t)M), c = (long)(e / (size_t)M);
    const size_t t = ((size_t)(r / NB) + (size_t)(c / NB) * MT) * NB * NB + (size_t)(c % NB) * NB + (r % NB);
    out[(size_t)c * ld + r] = T[t];
  }
}

__global__ void k_max_col_abs_sum(const double* X, long M, long N, unsigned long long* out_bits) {
  for (long c = blockIdx.x; c < N; c += gridDim.x) {
    double s = 0.0;
    for (long r = threadIdx.x; r < M; r += blockDim.x) s += fabs(X[(size_t)c * M + r]);
    s = warp_sum(s);
    __shared__ double red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[i];
      // non-negative doubles order like their bit patterns; NaN (all ones
      // exponent, non-zero mantissa) sorts above +inf and so propagates.
      atomicMax(out_bits, (unsigned long long)__double_as_longlong(t));
    }
    __syncthreads();
  }
}

// FP64 FMA issue-rate probe: the roofline denominator of the FP64 tile kernels
// (independent FMA chains, no memory traffic).
constexpr int kPeakIter = 2048;
__global__ void k_fp64_peak(double* out, double b, double c) {
  double a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5,
         a6 = a0 + 6, a7 = a0 + 7;
  for (int i = 0; i < kPeakIter; i++) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

// FP64 tensor-core (DMMA) issue-rate probe: mma.sync f64 on independent
// accumulators, no memory traffic.  SHAPE 0: m8n8k4 (A 1, B 1, C 2 doubles per
// thread); 1: m16n8k16 (A 8, B 4, C 4).
constexpr int kMmaIter = 1024;
constexpr int kMmaAcc = 4;
template <int SHAPE>
__global__ void __launch_bounds__(256) k_fp64_mma_peak(double* out, double av, double bv) {
  double a[8], b[4], d[kMmaAcc][4];
#pragma unroll
  for (int i = 0; i < 8; i++) a[i] = av * (threadIdx.x + i);
#pragma unroll
  for (int i = 0; i < 4; i++) b[i] = bv * (i + 1);
#pragma unroll
  for (int q = 0; q < kMmaAcc; q++)
#pragma unroll
    for (int i = 0; i < 4; i++) d[q][i] = 0.0;
  for (int it = 0; it < kMmaIter; it++) {
#pragma unroll
    for (int q = 0; q < kMmaAcc; q++) {
      if (SHAPE == 0) {
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                     : "+d"(d[q][0]), "+d"(d[q][1])
                     : "d"(a[q]), "d"(b[q]));
      } else {
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
            "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};"
            : "+d"(d[q][0]), "+d"(d[q][1]), "+d"(d[q][2]), "+d"(d[q][3])
            : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]), "d"(a[5]), "d"(a[6]), "d"(a[7]),
              "d"(b[0]), "d"(b[1]), "d"(b[2]), "d"(b[3]));
      }
    }
  }
  double t = 0.0;
#pragma unroll
  for (int q = 0; q < kMmaAcc; q++)
#pragma unroll
    for (int i = 0; i < 4; i++) t += d[q][i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = t;
}

double measure_fp64_mma_peak_tflops(int shape, cudaStream_t s) {
  if (shape != 0 && shape != 1) return -1.0;
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = nsm * 4, threads = 256;
  double* out = nullptr;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return -1.0;
  auto launch = [&]() {
    if (shape == 0)
      k_fp64_mma_peak<0><<<blocks, threads, 0, s>>>(out, 1e-3, 1e-3);
    else
      k_fp64_mma_peak<1><<<blocks, threads, 0, s>>>(out, 1e-3, 1e-3);
  };
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch();   // warm-up
  cudaEventRecord(e0, s);
  const int reps = 5;
  for (int r = 0; r < reps; r++) launch();
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  // flops per warp instruction: 2 m n k
  const double per_mma = shape == 0 ? 2.0 * 8 * 8 * 4 : 2.0 * 16 * 8 * 16;
  const double flops = (double)reps * blocks * (threads / 32) * kMmaIter * kMmaAcc * per_mma;
  return ms > 0 ? flops / (ms * 1e-3) / 1e12 : -1.0;
}

double measure_fp64_peak_tflops(cudaStream_t s) {
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = nsm * 8, threads = 256;
  double* out = nullptr;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_peak<<<blocks, threads, 0, s>>>(out, 1.0000001, 1e-9);   // warm-up
  cudaEventRecord(e0, s);
  const int reps = 5;
  for (int r = 0; r < reps; r++) k_fp64_peak<<<blocks, threads, 0, s>>>(out, 1.0000001, 1e-9);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double flops = (double)reps * blocks * threads * kPeakIter * 8 * 2.0;
  return ms > 0 ? flops / (ms * 1e-3) / 1e12 : -1.0;
}

static int grid_for(size_t n) {
  size_t g = (n + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  return (int)(g ? g : 1);
}

void fill_uniform(double* dA, long M, long N, int NB, uint64_t seed, cudaStream_t s) {
  k_fill_uniform<<<grid_for((size_t)M * N), 256, 0, s>>>(dA, M, N, NB, seed);
}
void make_identity(double* dQ, long M, long N, int NB, bool zero_first, cudaStream_t s) {
  k_identity<<<grid_for((size_t)M * N), 256, 0, s>>>(dQ, M, N, NB, zero_first ? 1 : 0);
}
void transpose_tiles(double* dQ, long N, int NB, cudaStream_t s) {
  const int nb = (int)(N / 32);
  k_transpose_tiles<<<dim3(nb, nb), dim3(32, 8), 0, s>>>(dQ, N, NB);
}
// Device address of host array h[0, n) when all of it is page-locked memory
// mapped into the device's address space, else null (pageable memory).
static double* mapped_range(const double* h, size_t n) {
  if (!h || n == 0) return nullptr;
  cudaPointerAttributes a{}, b{};
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess || a.type != cudaMemoryTypeHost || !a.devicePointer) {
    cudaGetLastError();
    return nullptr;
  }
  if (cudaPointerGetAttributes(&b, h + (n - 1)) != cudaSuccess || b.type != cudaMemoryTypeHost ||
      static_cast<double*>(b.devicePointer) != static_cast<double*>(a.devicePointer) + (n - 1)) {
    cudaGetLastError();
    return nullptr;
  }
  return static_cast<double*>(a.devicePointer);
}

static int copy_blocks() {
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return 4 * nsm;
}

static int aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0 ? 1 : 0; }

cudaError_t copy_host_to_device(double* d, const double* h, size_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  double* m = mapped_range(h, n);
  if (!m) return cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, s);
  k_copy_stream<<<copy_blocks(), 256, 0, s>>>(d, m, n, aligned16(d) & aligned16(m));
  return cudaGetLastError();
}

cudaError_t copy_device_to_host(double* h, const double* d, size_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  double* m = mapped_range(h, n);
  if (!m) return cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, s);
  k_copy_stream<<<copy_blocks(), 256, 0, s>>>(m, d, n, aligned16(d) & aligned16(m));
  return cudaGetLastError();
}

void zero_reflectors(double* dA, long M, long N, int NB, cudaStream_t s) {
  k_zero_reflectors<<<grid_for((size_t)M * N), 256, 0, s>>>(dA, M, N, NB);
}
void dgemm_tn_tiles(const double* dA, const double* dB, double* dC, long M, long N, int NB,
                    cudaStream_t s) {
  const int NT = (int)(N / NB);
  const int bpt = NB / kGB > 0 ? NB / kGB : 1;
  dim3 grid(NT * bpt, NT * bpt);
  k_dgemm_tn<<<grid, 256, 0, s>>>(dA, dB, dC, M, N, NB);
}
void frob_diff(const double* dX, const double* dY, double alpha_identity, long M, long N, int NB,
               double* d_out, cudaStream_t s) {
  cudaMemsetAsync(d_out, 0, sizeof(double), s);
  k_frob_diff<<<grid_for((size_t)M * N), 256, 0, s>>>(dX, dY, alpha_identity, M, N, NB, d_out);
}
void tiles_to_colmajor(const double* dT, double* dOut, long M, long N, int NB, cudaStream_t s) {
  k_tiles_to_colmajor<<<grid_for((size_t)M * N), 256, 0, s>>>(dT, dOut, M, N, NB, 1);
}
void colmajor_to_tiles(const double* dIn, double* dT, long M, long N, int NB, cudaStream_t s) {
  k_tiles_to_colmajor<<<grid_for((size_t)M * N), 256, 0, s>>>(dIn, dT, M, N, NB, 0);
}
void colmajor_to_tiles_padded(const double* dIn, long ld, long M, long N, int NB, double* dT, cudaStream_t s) {
  const int MT = (int)((M + NB - 1) / NB), NT = (int)((N + NB - 1) / NB);
  k_colmajor_to_tiles_padded<<<grid_for((size_t)MT * NT * NB * NB), 256, 0, s>>>(dIn, ld, M, N, NB, MT, NT, dT);
}
void tiles_to_colmajor_padded(const double* dT, long ld, long M, long N, int NB, double* dOut, cudaStream_t s) {
  const int MT = (int)((M + NB - 1) / NB);
  k_tiles_to_colmajor_padded<<<grid_for((size_t)M * N), 256, 0, s>>>(dT, ld, M, N, NB, MT, dOut);
}
void max_col_abs_sum(const double* dColMajor, long M, long N, double* d_out, cudaStream_t s) {
  cudaMemsetAsync(d_out, 0, sizeof(double), s);
  int g = (int)(N < 152 * 8 ? N : 152 * 8);
  k_max_col_abs_sum<<<g > 0 ? g : 1, 256, 0, s>>>(dColMajor, M, N, (unsigned long long*)d_out);
}

}  // namespace hqr
