// hqr_lstsq.cu -- device kernels of the least-squares solve (hqr_lstsq): the
// right-hand sides in and out of the tile layout, the FP64 residual
// r = b - A x on the original A, and the blocked back substitution with the R
// of a tile QR.
//
// The reference has no solve (its driver stops at Q and R, main.c:145-258);
// this is the first extension its callers need: x = R^-1 (Q^T b)(1:n), then
// FP64 iterative refinement x += R^-1 (Q^T (b - A x))(1:n).
#include "hqr_internal.h"

namespace hqr {
namespace {

constexpr int kRhsChunk = 16;   // right-hand sides per thread pass
constexpr int kRBlock = 32;     // columns of R staged per pass of the diagonal solve

// C (tile layout of an M x CT*NB matrix, MT tile rows) <- B (column-major
// nrows x nrhs, ld ldb), zero beyond column nrhs and row nrows.
__global__ void k_pack_rhs(const double* __restrict__ B, long ldb, int nrhs, long nrows, double* __restrict__ C,
                           long M, int MT, int NB, int CT) {
  const long n = M * (long)CT * NB;
  const long tile_elems = (long)NB * NB;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const long tile = e / tile_elems;
    const int within = (int)(e - tile * tile_elems);
    const long row = (tile % MT) * NB + within % NB;
    const long col = (tile / MT) * NB + within / NB;
    C[e] = (col < nrhs && row < nrows) ? B[row + col * ldb] : 0.0;
  }
}

// F -= R (column-major M x nrhs, leading dimensions ldf, ldr).
__global__ void k_sub_cm(double* __restrict__ F, long ldf, const double* __restrict__ R, long ldr, long M,
                         int nrhs) {
  const long n = M * (long)nrhs;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const long row = e % M, col = e / M;
    F[row + col * ldf] -= R[row + col * ldr];
  }
}

// R (column-major M x nrhs) += the first nrhs columns of D (tile layout, MT
// tile rows).
__global__ void k_add_unpack(double* __restrict__ R, long ldr, const double* __restrict__ D, long M, int MT,
                             int NB, int nrhs) {
  const long n = M * (long)nrhs;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const long row = e % M, col = e / M;
    R[row + col * ldr] += D[((row / NB) + (col / NB) * (long)MT) * NB * NB + (col % NB) * NB + row % NB];
  }
}

// Tile rows [ti0, ti1) of the MT x CT tile grids: D <- C (sub = 0) or
// C <- C - D (sub = 1).
__global__ void k_tile_rows(double* __restrict__ C, double* __restrict__ D, int MT, int NB, int CT, int ti0,
                            int ti1, int sub) {
  const long tile = (long)NB * NB;
  const long per_col = (long)(ti1 - ti0) * tile;
  const long n = per_col * CT;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const long tj = e / per_col, within = e % per_col;
    const long off = (tj * MT + ti0) * tile + within;
    if (sub)
      C[off] -= D[off];
    else
      D[off] = C[off];
  }
}

// Partial sums of A^T R over tile-row slice blockIdx.z: P[z] (column-major
// N x nrhs) = sum over tile rows ti = z, z + S, ... of A(ti, :)^T R(ti rows, :).
// Block (tj, q0 / kRhsChunk, z); thread c = column c of tile column tj (NB
// threads) walks its own (contiguous) tile column; R's rows are staged.
__global__ void k_atr(const double* __restrict__ A, long M, long N, int NB, const double* __restrict__ R,
                      long ldr, double* __restrict__ P, int nrhs) {
  extern __shared__ double sr[];   // NB x kRhsChunk rows of R
  const int MT = (int)(M / NB), S = (int)gridDim.z;
  const int tj = blockIdx.x, q0 = blockIdx.y * kRhsChunk, z = blockIdx.z;
  const int c = threadIdx.x;
  double acc[kRhsChunk];
#pragma unroll
  for (int q = 0; q < kRhsChunk; q++) acc[q] = 0.0;
  for (int ti = z; ti < MT; ti += S) {
    __syncthreads();
    for (int e = threadIdx.x; e < NB * kRhsChunk; e += blockDim.x) {
      const int k = e % NB, q = e / NB;
      sr[e] = (q0 + q < nrhs) ? R[(long)ti * NB + k + (long)(q0 + q) * ldr] : 0.0;
    }
    __syncthreads();
    const double* Ac = A + ((long)ti + (long)tj * MT) * NB * NB + (long)c * NB;
#pragma unroll 4
    for (int k = 0; k < NB; k++) {
      const double a = __ldg(Ac + k);
#pragma unroll
      for (int q = 0; q < kRhsChunk; q++) acc[q] = fma(a, sr[k + q * NB], acc[q]);
    }
  }
  double* Pz = P + (long)z * N * nrhs;
  const long row = (long)tj * NB + c;
#pragma unroll
  for (int q = 0; q < kRhsChunk; q++)
    if (q0 + q < nrhs) Pz[row + (long)(q0 + q) * N] = acc[q];
}

// G (column-major N x nrhs, ld ldg) = alpha * sum_z P[z], z in order.
__global__ void k_sum_partials(const double* __restrict__ P, int S, long N, int nrhs, double alpha,
                               double* __restrict__ G, long ldg) {
  const long n = N * (long)nrhs;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < S; z++) s += P[(long)z * n + e];
    G[(e % N) + (e / N) * ldg] = alpha * s;
  }
}

// X (column-major N x nrhs, ld ldx) <- Y or X + Y, Y = the first N rows of C
// (tile layout, MT tile rows).
__global__ void k_update_x(const double* __restrict__ C, int MT, int NB, long N, int nrhs,
                           double* __restrict__ X, long ldx, int accumulate) {
  const long n = N * (long)nrhs;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const long row = e % N, col = e / N;
    const long off = ((row / NB) + (col / NB) * (long)MT) * NB * NB + (col % NB) * NB + row % NB;
    const double y = C[off];
    X[row + col * ldx] = accumulate ? X[row + col * ldx] + y : y;
  }
}

// R = B - A X in FP64.  A: tile layout M x N; X: column-major N x nrhs;
// B, R: column-major M x nrhs.  Block (ti, q0 / kRhsChunk): tile row ti,
// right-hand sides q0..q0+15; thread r = row r of the tile row (NB threads).
__global__ void k_residual(const double* __restrict__ A, long M, long N, int NB,
                           const double* __restrict__ X, long ldx, const double* __restrict__ B,
                           long ldb, double* __restrict__ R, long ldr, int nrhs) {
  extern __shared__ double sx[];   // NB x kRhsChunk slice of X
  const int MT = (int)(M / NB), NT = (int)(N / NB);
  const int ti = blockIdx.x, q0 = blockIdx.y * kRhsChunk;
  const int r = threadIdx.x;
  double acc[kRhsChunk];
#pragma unroll
  for (int q = 0; q < kRhsChunk; q++) acc[q] = 0.0;
  for (int tj = 0; tj < NT; tj++) {
    __syncthreads();
    for (int e = threadIdx.x; e < NB * kRhsChunk; e += blockDim.x) {
      const int k = e % NB, q = e / NB;
      sx[e] = (q0 + q < nrhs) ? X[(long)tj * NB + k + (long)(q0 + q) * ldx] : 0.0;
    }
    __syncthreads();
    const double* At = A + ((long)ti + (long)tj * MT) * NB * NB;
#pragma unroll 4
    for (int k = 0; k < NB; k++) {
      const double a = __ldcs(At + r + (long)k * NB);
#pragma unroll
      for (int q = 0; q < kRhsChunk; q++) acc[q] = fma(a, sx[k + q * NB], acc[q]);
    }
  }
  const long row = (long)ti * NB + r;
#pragma unroll
  for (int q = 0; q < kRhsChunk; q++)
    if (q0 + q < nrhs) R[row + (long)(q0 + q) * ldr] = B[row + (long)(q0 + q) * ldb] - acc[q];
}

// ||R(:, q)||_2^2 of each column (column-major M x nrhs, ld ldr): one block per
// column, fixed summation order.
__global__ void k_col_norm2(const double* __restrict__ R, long M, long ldr, double* __restrict__ out) {
  __shared__ double red[32];
  const double* c = R + (long)blockIdx.x * ldr;
  double s = 0.0;
  for (long i = threadIdx.x; i < M; i += blockDim.x) s = fma(c[i], c[i], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    out[blockIdx.x] = t;
  }
}

// The two triangular solves give each block ONE right-hand side: FP64 issues
// at about one warp instruction per 70 cycles per SM sub-partition on this
// part, so a block that carried several columns through the serial diagonal
// solve spent most of each step there; one column per block spreads a step
// over nrhs times more SMs.  The diagonal solve multiplies by the reciprocal
// of each diagonal element, taken once per row by its own thread.
//
// One step of the back substitution R Y = C over the first NT tile rows of C
// (tile layout, MT tile rows), right-hand side q = blockIdx.y: step i < NT
// first updates blocks k < i, C_k -= R_ki Y_i (Y_i solved by the step before),
// then block k = i - 1 solves R_kk Y_k = C_k in place; step NT only solves
// block NT - 1.  RA: the factored A (R in its upper tiles).  Thread r owns
// row r of the tile (NB threads).
__global__ void k_trsm_step(const double* __restrict__ RA, int MT, int NB, double* __restrict__ C,
                            int i, int NT) {
  extern __shared__ double sm[];   // NB values of Y_i / NB x kRBlock columns of R_kk + 2
  const int k = (i < NT) ? (int)blockIdx.x : NT - 1;
  const int q = blockIdx.y, tj = q / NB, cw = q % NB;
  const int r = threadIdx.x;
  const long tile = (long)NB * NB;
  double* Ck = C + ((long)k + (long)tj * MT) * tile + (long)cw * NB;
  if (i < NT) {
    const double* Rki = RA + ((long)k + (long)i * MT) * tile;
    sm[r] = C[((long)i + (long)tj * MT) * tile + (long)cw * NB + r];
    __syncthreads();
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    for (int kk = 0; kk < NB; kk += 4) {
      a0 = fma(Rki[r + (long)kk * NB], sm[kk], a0);
      a1 = fma(Rki[r + (long)(kk + 1) * NB], sm[kk + 1], a1);
      a2 = fma(Rki[r + (long)(kk + 2) * NB], sm[kk + 2], a2);
      a3 = fma(Rki[r + (long)(kk + 3) * NB], sm[kk + 3], a3);
    }
    Ck[r] -= (a0 + a1) + (a2 + a3);
  }
  if (k != ((i < NT) ? i - 1 : NT - 1) || k < 0) return;
  // R_kk y = c_k from the bottom row: the solved value of row j is broadcast
  // through a double buffer (one barrier per row); R's columns are staged
  // kRBlock at a time (sR[rr + cc NB] = R(rr, jb + cc)).
  __syncthreads();
  const double* Rkk = RA + ((long)k + (long)k * MT) * tile;
  double* sR = sm;
  double* sy = sm + (long)NB * kRBlock;
  double v = Ck[r];
  const double inv = 1.0 / Rkk[r + (long)r * NB];
  int buf = 0;
  for (int jend = NB; jend > 0; jend -= kRBlock) {
    const int jb = jend > kRBlock ? jend - kRBlock : 0;
    __syncthreads();
    for (int e = threadIdx.x; e < NB * (jend - jb); e += blockDim.x)
      sR[e] = Rkk[(e % NB) + (long)(jb + e / NB) * NB];
    __syncthreads();
    for (int j = jend - 1; j >= jb; j--) {
      if (r == j) {
        v *= inv;
        sy[buf] = v;
      }
      __syncthreads();
      if (r < j) v = fma(-sR[r + (j - jb) * NB], sy[buf], v);
      buf ^= 1;
    }
  }
  Ck[r] = v;
}

// One step of the forward substitution R^T Y = C over the first NT tile rows
// of C, right-hand side q = blockIdx.y: step i first updates blocks k >= i,
// C_k -= R_(i-1)k^T Y_(i-1) (none at i = 0), then block k = i solves
// R_ii^T Y_i = C_i in place (R_ii^T lower triangular).  Row r of
// R_(i-1)k^T is column r of R_(i-1)k, contiguous in the tile.
__global__ void k_trsmt_step(const double* __restrict__ RA, int MT, int NB, double* __restrict__ C, int i) {
  extern __shared__ double sm[];   // NB values of Y_(i-1) / kRBlock x NB rows of R_kk + 2
  const int k = i + (int)blockIdx.x;
  const int q = blockIdx.y, tj = q / NB, cw = q % NB;
  const int r = threadIdx.x;
  const long tile = (long)NB * NB;
  double* Ck = C + ((long)k + (long)tj * MT) * tile + (long)cw * NB;
  if (i > 0) {
    const double* Rc = RA + ((long)(i - 1) + (long)k * MT) * tile + (long)r * NB;
    sm[r] = C[((long)(i - 1) + (long)tj * MT) * tile + (long)cw * NB + r];
    __syncthreads();
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    for (int kk = 0; kk < NB; kk += 4) {
      a0 = fma(Rc[kk], sm[kk], a0);
      a1 = fma(Rc[kk + 1], sm[kk + 1], a1);
      a2 = fma(Rc[kk + 2], sm[kk + 2], a2);
      a3 = fma(Rc[kk + 3], sm[kk + 3], a3);
    }
    Ck[r] -= (a0 + a1) + (a2 + a3);
  }
  if (k != i) return;
  // R_kk^T y = c_k from the top row; sR[(j - jb) + r kRBlock] = R(j, r).
  __syncthreads();
  const double* Rkk = RA + ((long)k + (long)k * MT) * tile;
  double* sR = sm;
  double* sy = sm + (long)NB * kRBlock;
  double v = Ck[r];
  const double inv = 1.0 / Rkk[r + (long)r * NB];
  int buf = 0;
  for (int jb = 0; jb < NB; jb += kRBlock) {
    const int je = min(NB, jb + kRBlock);
    __syncthreads();
    for (int e = threadIdx.x; e < (je - jb) * NB; e += blockDim.x) {
      const int jj = e % (je - jb), cc = e / (je - jb);
      sR[jj + cc * kRBlock] = Rkk[(jb + jj) + (long)cc * NB];
    }
    __syncthreads();
    for (int j = jb; j < je; j++) {
      if (r == j) {
        v *= inv;
        sy[buf] = v;
      }
      __syncthreads();
      if (r > j) v = fma(-sR[(j - jb) + r * kRBlock], sy[buf], v);
      buf ^= 1;
    }
  }
  Ck[r] = v;
}

int blocks_for(long n) {
  long b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 4 * 152 ? 4 * 152 : b));
}

}  // namespace

void pack_rhs(const double* dB, long ldb, int nrhs, double* dC, long M, int NB, int CT, cudaStream_t s) {
  k_pack_rhs<<<blocks_for(M * (long)CT * NB), 256, 0, s>>>(dB, ldb, nrhs, M, dC, M, (int)(M / NB), NB, CT);
}

void pack_rhs_rows(const double* dB, long ldb, int nrhs, long nrows, double* dC, long M, int NB, int CT,
                   cudaStream_t s) {
  k_pack_rhs<<<blocks_for(M * (long)CT * NB), 256, 0, s>>>(dB, ldb, nrhs, nrows, dC, M, (int)(M / NB), NB, CT);
}

void sub_colmajor(double* dF, long ldf, const double* dR, long ldr, long M, int nrhs, cudaStream_t s) {
  k_sub_cm<<<blocks_for(M * (long)nrhs), 256, 0, s>>>(dF, ldf, dR, ldr, M, nrhs);
}

void add_unpack(double* dR, long ldr, const double* dD, long M, int NB, int nrhs, cudaStream_t s) {
  k_add_unpack<<<blocks_for(M * (long)nrhs), 256, 0, s>>>(dR, ldr, dD, M, (int)(M / NB), NB, nrhs);
}

void tile_rows(double* dC, double* dD, long M, int NB, int CT, int ti0, int ti1, bool sub, cudaStream_t s) {
  if (ti1 <= ti0) return;
  k_tile_rows<<<blocks_for((long)(ti1 - ti0) * NB * NB * CT), 256, 0, s>>>(dC, dD, (int)(M / NB), NB, CT, ti0,
                                                                            ti1, sub ? 1 : 0);
}

int atr_slices(long M, long N, int NB, int nrhs) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long base = (N / NB) * ((nrhs + kRhsChunk - 1) / kRhsChunk);
  const long want = (4L * sms + base - 1) / base;
  return (int)(want < 1 ? 1 : (want > M / NB ? M / NB : want));
}

int at_times(const double* dA, long M, long N, int NB, const double* dR, long ldr, int nrhs, double alpha,
             double* dG, long ldg, double* dP, int S, cudaStream_t s) {
  const dim3 grid((unsigned)(N / NB), (unsigned)((nrhs + kRhsChunk - 1) / kRhsChunk), (unsigned)S);
  const size_t smem = (size_t)NB * kRhsChunk * sizeof(double);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_atr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return record_cuda_error(e, "cudaFuncSetAttribute(k_atr)");
  }
  k_atr<<<grid, NB, smem, s>>>(dA, M, N, NB, dR, ldr, dP, nrhs);
  k_sum_partials<<<blocks_for(N * (long)nrhs), 256, 0, s>>>(dP, S, N, nrhs, alpha, dG, ldg);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? HQR_OK : record_cuda_error(e, "k_atr launch");
}

void update_x(const double* dC, long M, int NB, long N, int nrhs, double* dX, long ldx, bool accumulate,
              cudaStream_t s) {
  k_update_x<<<blocks_for(N * (long)nrhs), 256, 0, s>>>(dC, (int)(M / NB), NB, N, nrhs, dX, ldx,
                                                         accumulate ? 1 : 0);
}

int residual(const double* dA, long M, long N, int NB, const double* dX, long ldx, const double* dB,
             long ldb, double* dR, long ldr, int nrhs, cudaStream_t s) {
  const dim3 grid((unsigned)(M / NB), (unsigned)((nrhs + kRhsChunk - 1) / kRhsChunk));
  const size_t smem = (size_t)NB * kRhsChunk * sizeof(double);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_residual, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return record_cuda_error(e, "cudaFuncSetAttribute(k_residual)");
  }
  k_residual<<<grid, NB, smem, s>>>(dA, M, N, NB, dX, ldx, dB, ldb, dR, ldr, nrhs);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? HQR_OK : record_cuda_error(e, "k_residual launch");
}

void col_norm2(const double* dR, long M, long ldr, int nrhs, double* dOut, cudaStream_t s) {
  k_col_norm2<<<nrhs, 256, 0, s>>>(dR, M, ldr, dOut);
}

size_t trsm_smem_bytes(int NB) { return ((size_t)NB * kRBlock + 2) * sizeof(double); }

int trsm_tiles(const double* dRA, long M, long N, int NB, double* dC, int nrhs, cudaStream_t s) {
  const int MT = (int)(M / NB), NT = (int)(N / NB);
  const size_t smem = trsm_smem_bytes(NB);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_trsm_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return record_cuda_error(e, "cudaFuncSetAttribute(k_trsm_step)");
  }
  for (int i = NT; i >= 1; i--) {
    const dim3 grid((unsigned)(i < NT ? i : 1), (unsigned)nrhs);
    k_trsm_step<<<grid, NB, smem, s>>>(dRA, MT, NB, dC, i, NT);
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? HQR_OK : record_cuda_error(e, "k_trsm_step launch");
}

int trsmt_tiles(const double* dRA, long M, long N, int NB, double* dC, int nrhs, cudaStream_t s) {
  const int MT = (int)(M / NB), NT = (int)(N / NB);
  const size_t smem = trsm_smem_bytes(NB);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_trsmt_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return record_cuda_error(e, "cudaFuncSetAttribute(k_trsmt_step)");
  }
  for (int i = 0; i < NT; i++) {
    const dim3 grid((unsigned)(NT - i), (unsigned)nrhs);
    k_trsmt_step<<<grid, NB, smem, s>>>(dRA, MT, NB, dC, i);
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? HQR_OK : record_cuda_error(e, "k_trsmt_step launch");
}

}  // namespace hqr
