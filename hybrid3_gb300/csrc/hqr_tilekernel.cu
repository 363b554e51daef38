// hqr_tilekernel.cu -- the reference's per-tile kernels (tile_kernel.h:28-230,
// bodies tile_kernel.c:19-716) with their own conventions, on the GPU.
//
// Each entry point runs one CTA of kThreads FP64 threads on one tile (or tile
// pair) in device memory.  Host pointers are staged through a device scratch
// pool for the call (copied in, and back out for every array the function may
// write); device and managed pointers are used in place.  The calls are
// synchronous, like the reference's.  Conventions (which differ from the
// LAPACK-style factorization path):
//   * reflector (tile_kernel.c:138-218): beta = +sqrt(alpha^2 + ||x||^2),
//     y_head = alpha - beta, t = 2 / (y_head^2 + ||x||^2), v = x / y_head,
//     tau = t * y_head^2; no guard for a zero column;
//   * T lower triangular: T(i,i) = tau_i, T(i,0:i) = -tau_i (T(0:i,0:i)^T
//     (Y^T y_i)(0:i)) (tile_kernel.c:220-262), T's strict upper part read as
//     stored;
//   * application (tile_kernel.c:264-363): W = Y^T A (Y lower, its stored
//     diagonal used), W = T W, A -= Y W.
// The reference's quirks are kept and listed at each function.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "hqr_common.cuh"
#include "hqr_internal.h"
#include "tile_kernel.h"

namespace hqr {
namespace tk {

// ---------------------------------------------------------------------------
// Device kernels (one CTA each)
// ---------------------------------------------------------------------------

// out[c] = sum_{r < n} x[r] * (base + c*ld)[r] for c < nc: one warp per column.
__device__ void col_dots(const double* x, const double* base, int ld, int n, int nc, double* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int c = warp; c < nc; c += kWarps) {
    const double* y = base + (size_t)c * ld;
    double s = 0.0;
    for (int r = lane; r < n; r += 32) s = fma(x[r], y[r], s);
    s = warp_sum(s);
    if (lane == 0) out[c] = s;
  }
}

// tile_sub_dgeqr2 (tile_kernel.c:138-218).  Quirks: no zero-norm guard; with
// row == col, TAU[col-1] is left unwritten and Y(col-1,col-1) is set to 0.
// Dynamic shared memory: col doubles.
__global__ void __launch_bounds__(kThreads) k_sub_dgeqr2(int row, int col, double* A, int lda, double* TAU,
                                                          double* Y) {
  extern __shared__ double yA[];
  __shared__ double sc[3];
  const int tid = threadIdx.x;
  int i;
  for (i = 0; i < col - 1; i++) {
    double* aii = A + i + (size_t)lda * i;
    col_dots(aii + 1, aii + 1, lda, row - i - 1, col - i, yA);
    __syncthreads();
    if (tid == 0) {
      const double a_head = aii[0], norm_1 = yA[0];
      const double norm = norm_1 + a_head * a_head;
      const double b = sqrt(norm);
      const double y_head = a_head - b;
      aii[0] = y_head;
      sc[0] = b;
      sc[1] = y_head;
      sc[2] = 2.0 / (y_head * y_head + norm_1);
    }
    __syncthreads();
    const double b = sc[0], y_head = sc[1], t = sc[2];
    for (int c = tid; c < col - i - 1; c += kThreads) yA[1 + c] += y_head * A[i + (size_t)lda * (i + 1 + c)];
    __syncthreads();
    const int nr = row - i, nc = col - i - 1;
    for (int e = tid; e < nr * nc; e += kThreads) {
      const int r = e % nr, c = e / nr;
      A[i + r + (size_t)lda * (i + 1 + c)] += -t * aii[r] * yA[1 + c];
    }
    __syncthreads();
    const double inv = 1.0 / y_head;
    for (int r = tid; r < row - i - 1; r += kThreads) {
      const double v = aii[1 + r] * inv;
      aii[1 + r] = v;
      Y[i + (size_t)lda * i + 1 + r] = v;
    }
    if (tid == 0) {
      aii[0] = b;
      Y[i + (size_t)lda * i] = 1.0;
      TAU[i] = t * y_head * y_head;
    }
    __syncthreads();
  }
  if (col <= 0) return;
  i = col - 1;
  if (row > col) {
    double* aii = A + i + (size_t)lda * i;
    col_dots(aii + 1, aii + 1, lda, row - i - 1, 1, yA);
    __syncthreads();
    if (tid == 0) {
      const double a_head = aii[0], norm_1 = yA[0];
      const double norm = norm_1 + a_head * a_head;
      const double b = sqrt(norm);
      const double y_head = a_head - b;
      aii[0] = b;
      sc[1] = y_head;
      sc[2] = 2.0 / (y_head * y_head + norm_1);
    }
    __syncthreads();
    const double y_head = sc[1], t = sc[2];
    const double inv = 1.0 / y_head;
    for (int r = tid; r < row - i - 1; r += kThreads) {
      const double v = aii[1 + r] * inv;
      aii[1 + r] = v;
      Y[i + (size_t)lda * i + 1 + r] = v;
    }
    if (tid == 0) {
      Y[i + (size_t)lda * i] = 1.0;
      TAU[i] = t * y_head * y_head;
    }
  } else if (row == col && tid == 0) {
    Y[i + (size_t)lda * i] = 0.0;
  }
}

// tile_sub_dtsqr2 (tile_kernel.c:654-716): QR of [A1 (upper col x col); A2
// (row x col)], A2 becomes V.  Dynamic shared memory: col doubles.
__global__ void __launch_bounds__(kThreads) k_sub_dtsqr2(int row, int col, double* A1, int lda1, double* A2,
                                                          int lda2, double* TAU) {
  extern __shared__ double dv[];
  __shared__ double sc[3];
  const int tid = threadIdx.x;
  int i;
  for (i = 0; i < col - 1; i++) {
    double* v = A2 + (size_t)i * lda2;
    col_dots(v, v, lda2, row, col - i, dv);
    __syncthreads();
    if (tid == 0) {
      const double a_head = A1[i + (size_t)i * lda1], norm_1 = dv[0];
      const double norm = norm_1 + a_head * a_head;
      const double b = sqrt(norm);
      const double y_head = a_head - b;
      sc[0] = b;
      sc[1] = y_head;
      sc[2] = 2.0 / (y_head * y_head + norm_1);
    }
    __syncthreads();
    const double b = sc[0], y_head = sc[1], t = sc[2];
    for (int c = tid; c < col - i - 1; c += kThreads) {
      double* a1 = A1 + i + (size_t)(i + 1 + c) * lda1;
      const double d = dv[1 + c] + y_head * a1[0];
      dv[1 + c] = d;
      a1[0] += -t * y_head * d;
    }
    __syncthreads();
    const int nc = col - i - 1;
    for (int e = tid; e < row * nc; e += kThreads) {
      const int r = e % row, c = e / row;
      A2[r + (size_t)(i + 1 + c) * lda2] += -t * v[r] * dv[1 + c];
    }
    __syncthreads();
    const double inv = 1.0 / y_head;
    for (int r = tid; r < row; r += kThreads) v[r] *= inv;
    if (tid == 0) {
      A1[i + (size_t)i * lda1] = b;
      TAU[i] = t * y_head * y_head;
    }
    __syncthreads();
  }
  if (col <= 0) return;
  i = col - 1;
  double* v = A2 + (size_t)i * lda2;
  col_dots(v, v, lda2, row, 1, dv);
  __syncthreads();
  if (tid == 0) {
    const double a_head = A1[i + (size_t)i * lda1], norm_1 = dv[0];
    const double norm = norm_1 + a_head * a_head;
    const double b = sqrt(norm);
    const double y_head = a_head - b;
    A1[i + (size_t)i * lda1] = b;
    sc[1] = y_head;
    sc[2] = 2.0 / (y_head * y_head + norm_1);
  }
  __syncthreads();
  const double y_head = sc[1], t = sc[2];
  const double inv = 1.0 / y_head;
  for (int r = tid; r < row; r += kThreads) v[r] *= inv;
  if (tid == 0) TAU[i] = t * y_head * y_head;
}

// tile_sub_dlarft (tile_kernel.c:220-262): lower T (ld ldt) from Y (ld lda,
// all `row` rows as stored) and TAU.  G: col x col global scratch.
__global__ void __launch_bounds__(kThreads) k_sub_dlarft(int row, int col, const double* Y, int lda,
                                                          const double* TAU, double* T, int ldt, double* G,
                                                          int transpose_out) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // G(i, c) = Y(:,i)^T Y(:,c) for c < i
  const int npairs = col * (col - 1) / 2;
  for (int p = warp; p < npairs; p += kWarps) {
    int i = 1, base = 0;
    while (base + i <= p) {
      base += i;
      i++;
    }
    const int c = p - base;
    const double* yi = Y + (size_t)i * lda;
    const double* yc = Y + (size_t)c * lda;
    double s = 0.0;
    for (int r = lane; r < row; r += 32) s = fma(yi[r], yc[r], s);
    s = warp_sum(s);
    if (lane == 0) G[i + (size_t)c * col] = s;
  }
  for (int i = tid; i < col; i += kThreads) T[i + (size_t)i * ldt] = TAU[i];
  __syncthreads();
  for (int i = 1; i < col; i++) {
    const double alpha = -T[i + (size_t)i * ldt];
    for (int r = tid; r < i; r += kThreads) {
      double s = 0.0;
      for (int c = 0; c < i; c++) s = fma(T[c + (size_t)r * ldt], G[i + (size_t)c * col], s);
      T[i + (size_t)r * ldt] = alpha * s;
    }
    __syncthreads();
  }
  if (transpose_out) {
    // T holds the lower T here (a zeroed scratch); move it to the upper part
    for (int e = tid; e < col * col; e += kThreads) {
      const int r = e % col, c = e / col;
      if (r > c) {
        T[c + (size_t)r * ldt] = T[r + (size_t)c * ldt];
        T[r + (size_t)c * ldt] = 0.0;
      }
    }
  }
}

// tile_dlarft (tile_kernel.c:368-437) with 2 <= block < col: couples the
// existing diagonal blocks, reading T and Y row-major as the reference does
// (Trm(a,b) = T[a*ldt + b]).  G: col x ldg scratch, T1: col x block scratch.
__global__ void __launch_bounds__(kThreads) k_dlarft_block(int row, int col, int block, const double* Y,
                                                            int lda, double* T, int ldt, double* G, int ldg,
                                                            double* T1) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int p = warp; p < col * col; p += kWarps) {
    const int a = p / col, b = p % col;
    const double* ya = Y + (size_t)a * lda;
    const double* yb = Y + (size_t)b * lda;
    double s = 0.0;
    for (int r = lane; r < row; r += 32) s = fma(ya[r], yb[r], s);
    s = warp_sum(s);
    if (lane == 0) G[(size_t)a * ldg + b] = s;
  }
  __syncthreads();
  for (int i = block; i < col - block; i += block) {
    for (int e = tid; e < i * block; e += kThreads) {
      const int a = e / block, b = e % block;
      double s = 0.0;
      for (int q = 0; q < i; q++) s = fma(T[(size_t)a * ldt + q], G[(size_t)q * ldg + i + b], s);
      T1[(size_t)a * block + b] = s;
    }
    __syncthreads();
    for (int e = tid; e < i * block; e += kThreads) {
      const int a = e / block, b = e % block;
      double s = 0.0;
      for (int q = 0; q < block; q++) s = fma(T1[(size_t)a * block + q], T[(size_t)(i + q) * ldt + i + b], s);
      T[(size_t)a * ldt + i + b] = -s;
    }
    __syncthreads();
  }
  for (int i = (col / block) * block; i < col; i++) {
    const double alpha = -T[i + (size_t)i * ldt];
    for (int a = tid; a < i; a += kThreads) {
      double s = 0.0;
      for (int q = 0; q < i; q++) s = fma(T[(size_t)a * ldt + q], G[(size_t)q * ldg + i], s);
      T[(size_t)a * ldt + i] = alpha * s;
    }
    __syncthreads();
  }
}

// tile_sub_dlarfb (tile_kernel.c:264-311): A (row x A_col) <- A - Y T' (Y^T A)
// with Y lower (row x row, stored diagonal) for the product and Y's first
// Y_col columns as stored for the update; T' = T (lower) or, with transT, the
// transpose of T's lower part (tile_return_dlarfb, tile_kernel.c:501-601).
// D, D2: Y_col x A_col global scratch.
__global__ void __launch_bounds__(kThreads) k_sub_dlarfb(int row, int Y_col, int A_col, const double* Y,
                                                          int ldy, const double* T, int ldt, double* A, int lda,
                                                          double* D, double* D2, int transT) {
  const int tid = threadIdx.x;
  for (int e = tid; e < Y_col * A_col; e += kThreads) {
    const int r = e % Y_col, c = e / Y_col;
    double s = 0.0;
    for (int q = r; q < row; q++) s = fma(Y[q + (size_t)r * ldy], A[q + (size_t)c * lda], s);
    D[r + (size_t)c * Y_col] = s;
  }
  __syncthreads();
  for (int e = tid; e < Y_col * A_col; e += kThreads) {
    const int r = e % Y_col, c = e / Y_col;
    double s = 0.0;
    if (transT) {
      for (int q = r; q < Y_col; q++) s = fma(T[q + (size_t)r * ldt], D[q + (size_t)c * Y_col], s);
    } else {
      for (int q = 0; q <= r; q++) s = fma(T[r + (size_t)q * ldt], D[q + (size_t)c * Y_col], s);
    }
    D2[r + (size_t)c * Y_col] = s;
  }
  __syncthreads();
  for (int e = tid; e < row * A_col; e += kThreads) {
    const int r = e % row, c = e / row;
    double s = 0.0;
    for (int q = 0; q < Y_col; q++) s = fma(Y[r + (size_t)q * ldy], D2[q + (size_t)c * Y_col], s);
    A[r + (size_t)c * lda] -= s;
  }
}

// tile_sub_dssrfb (tile_kernel.c:313-363) and its pieces.
//   part 0: the whole update; 1: tile_dssrfb_head (A1 update, D kept in U,
//   ld over_row); 2: tile_dssrfb_tail (A2 -= Y D from U).
// Quirk kept: rows Y_col..over_row-1 of A1 are zeroed (A1 -= its own copy).
// transT: T read transposed (tile_return_dssrfb).  D: over_row x A_col, D2:
// Y_col x A_col global scratch.
__global__ void __launch_bounds__(kThreads) k_sub_dssrfb(int over_row, int under_row, int Y_col, int A_col,
                                                          const double* Y, int ldy, const double* T, int ldt,
                                                          double* A1, int lda1, double* A2, int lda2, double* D,
                                                          double* D2, double* U, int part, int transT) {
  const int tid = threadIdx.x;
  if (part != 2) {
    for (int e = tid; e < over_row * A_col; e += kThreads) {
      const int r = e % over_row, c = e / over_row;
      double d = A1[r + (size_t)c * lda1];
      if (r < Y_col) {
        double s = 0.0;
        for (int q = 0; q < under_row; q++) s = fma(Y[q + (size_t)r * ldy], A2[q + (size_t)c * lda2], s);
        d += s;
      }
      D[r + (size_t)c * over_row] = d;
    }
    __syncthreads();
    for (int e = tid; e < Y_col * A_col; e += kThreads) {
      const int r = e % Y_col, c = e / Y_col;
      double s = 0.0;
      if (transT) {
        for (int q = r; q < Y_col; q++) s = fma(T[q + (size_t)r * ldt], D[q + (size_t)c * over_row], s);
      } else {
        for (int q = 0; q <= r; q++) s = fma(T[r + (size_t)q * ldt], D[q + (size_t)c * over_row], s);
      }
      D2[r + (size_t)c * Y_col] = s;
    }
    __syncthreads();
    for (int e = tid; e < over_row * A_col; e += kThreads) {
      const int r = e % over_row, c = e / over_row;
      const double d = (r < Y_col) ? D2[r + (size_t)c * Y_col] : D[r + (size_t)c * over_row];
      A1[r + (size_t)c * lda1] -= d;
      if (part == 1) U[r + (size_t)c * over_row] = d;
    }
    if (part == 1) return;
    __syncthreads();
  }
  const double* W = (part == 2) ? U : D2;
  const int ldw = (part == 2) ? over_row : Y_col;
  for (int e = tid; e < under_row * A_col; e += kThreads) {
    const int r = e % under_row, c = e / under_row;
    double s = 0.0;
    for (int q = 0; q < Y_col; q++) s = fma(Y[r + (size_t)q * ldy], W[q + (size_t)c * ldw], s);
    A2[r + (size_t)c * lda2] -= s;
  }
}

// ---------------------------------------------------------------------------
// Host side: staging of host arrays, scratch, launches
// ---------------------------------------------------------------------------
std::mutex g_mu;                 // one tile call at a time (shared scratch)
double* g_scratch = nullptr;     // device scratch pool (grow-only)
size_t g_scratch_cap = 0;
cudaStream_t g_stream = nullptr;

// Elements spanned by a column-major rows x cols block with leading dimension ld.
size_t extent(int ld, int rows, int cols) {
  if (rows <= 0 || cols <= 0) return 0;
  return (size_t)(cols - 1) * (size_t)ld + (size_t)rows;
}

bool device_accessible(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();   // an unregistered host pointer: clear the error
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// The arrays of one call: device views of every argument, staged if needed.
class Call {
 public:
  explicit Call(const char* fn) : fn_(fn), lock_(g_mu) {}
  ~Call() { finish(); }
  // Register an array of n doubles; `out`: the function may write it.
  double* arg(const double* p, size_t n, bool out) {
    if (rc_ != HQR_OK || !p || n == 0) return const_cast<double*>(p);
    if (device_accessible(p)) return const_cast<double*>(p);
    if (nargs_ == kMaxArgs) {
      rc_ = HQR_ERR_INVALID;
      return nullptr;
    }
    Arg& a = args_[nargs_++];
    a.host = const_cast<double*>(p);
    a.n = n;
    a.out = out;
    a.off = used_;
    used_ += (n + 31) & ~size_t(31);
    return nullptr;   // resolved by bind()
  }
  // Scratch of n doubles (valid after bind()).
  size_t scratch(size_t n) {
    const size_t off = used_;
    used_ += (n + 31) & ~size_t(31);
    return off;
  }
  // Allocate the pool, copy the staged inputs in; returns the pool base.
  double* bind() {
    if (rc_ != HQR_OK) return nullptr;
    if (!g_stream && cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking) != cudaSuccess) {
      rc_ = record_cuda_error(cudaGetLastError(), fn_);
      return nullptr;
    }
    if (g_scratch_cap < used_) {
      if (g_scratch) cudaFree(g_scratch);
      g_scratch = nullptr;
      g_scratch_cap = 0;
      if (cudaMalloc(&g_scratch, used_ * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        rc_ = HQR_ERR_NOMEM;
        return nullptr;
      }
      g_scratch_cap = used_;
    }
    for (int i = 0; i < nargs_; i++) {
      const Arg& a = args_[i];
      if (cudaMemcpyAsync(g_scratch + a.off, a.host, a.n * sizeof(double), cudaMemcpyHostToDevice,
                          g_stream) != cudaSuccess) {
        rc_ = record_cuda_error(cudaGetLastError(), fn_);
        return nullptr;
      }
    }
    bound_ = true;
    return g_scratch;
  }
  // Device view of a registered array.
  double* view(const double* p, double* registered) const {
    if (registered || !p) return registered;
    for (int i = 0; i < nargs_; i++)
      if (args_[i].host == p) return g_scratch + args_[i].off;
    return nullptr;
  }
  cudaStream_t stream() const { return g_stream; }
  bool ok() const { return rc_ == HQR_OK; }
  void launched() {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess && rc_ == HQR_OK) rc_ = record_cuda_error(e, fn_);
  }

 private:
  struct Arg {
    double* host;
    size_t n, off;
    bool out;
  };
  static constexpr int kMaxArgs = 8;
  void finish() {
    if (bound_ && rc_ == HQR_OK) {
      for (int i = 0; i < nargs_; i++) {
        const Arg& a = args_[i];
        if (!a.out) continue;
        if (cudaMemcpyAsync(a.host, g_scratch + a.off, a.n * sizeof(double), cudaMemcpyDeviceToHost,
                            g_stream) != cudaSuccess) {
          rc_ = record_cuda_error(cudaGetLastError(), fn_);
          break;
        }
      }
    }
    if (bound_) {
      const cudaError_t e = cudaStreamSynchronize(g_stream);
      if (e != cudaSuccess && rc_ == HQR_OK) rc_ = record_cuda_error(e, fn_);
    }
    report_error(fn_, rc_);
  }
  const char* fn_;
  std::lock_guard<std::mutex> lock_;
  Arg args_[kMaxArgs];
  int nargs_ = 0;
  size_t used_ = 0;
  bool bound_ = false;
  int rc_ = HQR_OK;
};

// Launch helpers on device pointers (all sizes already validated).
void sub_dgeqr2(cudaStream_t s, int row, int col, double* A, int lda, double* TAU, double* Y) {
  k_sub_dgeqr2<<<1, kThreads, (size_t)(col > 0 ? col : 1) * sizeof(double), s>>>(row, col, A, lda, TAU, Y);
}
void sub_dtsqr2(cudaStream_t s, int row, int col, double* A1, int lda1, double* A2, int lda2, double* TAU) {
  k_sub_dtsqr2<<<1, kThreads, (size_t)(col > 0 ? col : 1) * sizeof(double), s>>>(row, col, A1, lda1, A2, lda2,
                                                                                   TAU);
}
void sub_dlarft(cudaStream_t s, int row, int col, const double* Y, int lda, const double* TAU, double* T, int ldt,
                double* G, int transpose_out) {
  k_sub_dlarft<<<1, kThreads, 0, s>>>(row, col, Y, lda, TAU, T, ldt, G, transpose_out);
}
void sub_dlarfb(cudaStream_t s, int row, int Y_col, int A_col, const double* Y, int ldy, const double* T, int ldt,
                double* A, int lda, double* D, double* D2, int transT) {
  k_sub_dlarfb<<<1, kThreads, 0, s>>>(row, Y_col, A_col, Y, ldy, T, ldt, A, lda, D, D2, transT);
}
void sub_dssrfb(cudaStream_t s, int over_row, int under_row, int Y_col, int A_col, const double* Y, int ldy,
                const double* T, int ldt, double* A1, int lda1, double* A2, int lda2, double* D, double* D2,
                double* U, int part, int transT) {
  k_sub_dssrfb<<<1, kThreads, 0, s>>>(over_row, under_row, Y_col, A_col, Y, ldy, T, ldt, A1, lda1, A2, lda2, D,
                                     D2, U, part, transT);
}

}  // namespace tk
}  // namespace hqr

using hqr::tk::Call;
using hqr::tk::extent;

extern "C" {

void* tile_init(char type, int tile_row, int tile_col) {
  (void)type;   // tile_kernel.c:19-25 allocates doubles whatever the type
  return calloc((size_t)tile_row * tile_col * 3, sizeof(double));
}

// tile_kernel.c:138-218.  row < col is rejected (HQR_ERR_INVALID): the
// reference's loop then walks the diagonal past the last row.
void tile_sub_dgeqr2(const int row, const int col, double* A, const int lda, double* TAU, double* Y,
                     double* work) {
  (void)work;
  if (row <= 0 || col <= 0) return;
  if (row < col || lda < row) {
    hqr::report_error("tile_sub_dgeqr2", HQR_ERR_INVALID);
    return;
  }
  Call call("tile_sub_dgeqr2");
  double* dA = call.arg(A, extent(lda, row, col), true);
  double* dT = call.arg(TAU, col, true);
  double* dY = call.arg(Y, extent(lda, row, col), true);
  if (!call.bind()) return;
  hqr::tk::sub_dgeqr2(call.stream(), row, col, call.view(A, dA), lda, call.view(TAU, dT), call.view(Y, dY));
  call.launched();
}

// tile_kernel.c:654-716
void tile_sub_dtsqr2(const int row, const int col, double* A1, const int lda1, double* A2, const int lda2,
                     double* TAU, double* work) {
  (void)work;
  if (row <= 0 || col <= 0) return;
  Call call("tile_sub_dtsqr2");
  double* d1 = call.arg(A1, extent(lda1, col, col), true);
  double* d2 = call.arg(A2, extent(lda2, row, col), true);
  double* dt = call.arg(TAU, col, true);
  if (!call.bind()) return;
  hqr::tk::sub_dtsqr2(call.stream(), row, col, call.view(A1, d1), lda1, call.view(A2, d2), lda2,
                      call.view(TAU, dt));
  call.launched();
}

// tile_kernel.c:220-262
void tile_sub_dlarft(const int row, const int col, const double* Y, const int lda, const double* TAU, double* T,
                     const int ldt, double* work) {
  (void)work;
  if (row <= 0 || col <= 0) return;
  Call call("tile_sub_dlarft");
  double* dy = call.arg(Y, extent(lda, row, col), false);
  double* dtau = call.arg(TAU, col, false);
  double* dT = call.arg(T, extent(ldt, col, col), true);
  const size_t g = call.scratch((size_t)col * col);
  double* base = call.bind();
  if (!base) return;
  hqr::tk::sub_dlarft(call.stream(), row, col, call.view(Y, dy), lda, call.view(TAU, dtau), call.view(T, dT), ldt,
                      base + g, 0);
  call.launched();
}

// tile_kernel.c:264-311
void tile_sub_dlarfb(const int row, const int Y_col, const int A_col, const double* Y, const int ldy,
                     const double* T, const int ldt, double* A, const int lda, double* work) {
  (void)work;
  if (row <= 0 || Y_col <= 0 || A_col <= 0) return;
  Call call("tile_sub_dlarfb");
  double* dy = call.arg(Y, extent(ldy, row, Y_col), false);
  double* dT = call.arg(T, extent(ldt, Y_col, Y_col), false);
  double* dA = call.arg(A, extent(lda, row, A_col), true);
  const size_t d = call.scratch((size_t)Y_col * A_col), d2 = call.scratch((size_t)Y_col * A_col);
  double* base = call.bind();
  if (!base) return;
  hqr::tk::sub_dlarfb(call.stream(), row, Y_col, A_col, call.view(Y, dy), ldy, call.view(T, dT), ldt,
                      call.view(A, dA), lda, base + d, base + d2, 0);
  call.launched();
}

// tile_kernel.c:313-363
void tile_sub_dssrfb(const int over_row, const int under_row, const int Y_col, const int A_col, const double* Y,
                     const int ldy, const double* T, const int ldt, double* A1, const int lda1, double* A2,
                     const int lda2, double* work) {
  (void)work;
  if (over_row <= 0 || under_row <= 0 || Y_col <= 0 || A_col <= 0) return;
  Call call("tile_sub_dssrfb");
  double* dy = call.arg(Y, extent(ldy, under_row, Y_col), false);
  double* dT = call.arg(T, extent(ldt, Y_col, Y_col), false);
  double* d1 = call.arg(A1, extent(lda1, over_row, A_col), true);
  double* d2 = call.arg(A2, extent(lda2, under_row, A_col), true);
  const size_t d = call.scratch((size_t)over_row * A_col), dd = call.scratch((size_t)Y_col * A_col);
  double* base = call.bind();
  if (!base) return;
  hqr::tk::sub_dssrfb(call.stream(), over_row, under_row, Y_col, A_col, call.view(Y, dy), ldy, call.view(T, dT),
                      ldt, call.view(A1, d1), lda1, call.view(A2, d2), lda2, base + d, base + dd, nullptr, 0, 0);
  call.launched();
}

// tile_kernel.c:28-57.  Quirk kept: only the diagonal T blocks are built.
void tile_dgeqrt(const int row, const int col, const int block, double* A, const int lda, double* TAU, double* Y,
                 double* T, const int ldt, double* work) {
  (void)work;
  if (row <= 0 || col <= 0 || block <= 0) return;
  if (row < col || lda < row || ldt < col) {   // as tile_sub_dgeqr2
    hqr::report_error("tile_dgeqrt", HQR_ERR_INVALID);
    return;
  }
  Call call("tile_dgeqrt");
  double* dA = call.arg(A, extent(lda, row, col), true);
  double* dtau = call.arg(TAU, col, true);
  double* dY = call.arg(Y, extent(lda, row, col), true);
  double* dT = call.arg(T, extent(ldt, col, col), true);
  const size_t g = call.scratch((size_t)col * col);
  const size_t d = call.scratch((size_t)row * col), d2 = call.scratch((size_t)row * col);
  double* base = call.bind();
  if (!base) return;
  A = call.view(A, dA);
  TAU = call.view(TAU, dtau);
  Y = call.view(Y, dY);
  T = call.view(T, dT);
  cudaStream_t s = call.stream();
  int i;
  for (i = 0; i < col - block; i += block) {
    hqr::tk::sub_dgeqr2(s, row - i, block, A + i * lda + i, lda, TAU + i, Y + i * lda + i);
    hqr::tk::sub_dlarft(s, row - i, block, Y + i * lda + i, lda, TAU + i, T + i * ldt + i, ldt, base + g, 0);
    hqr::tk::sub_dlarfb(s, row - i, block, col - i - block, Y + i * lda + i, lda, T + i * ldt + i, ldt,
                        A + (i + block) * lda + i, lda, base + d, base + d2, 0);
  }
  hqr::tk::sub_dgeqr2(s, row - i, col - i, A + i * lda + i, lda, TAU + i, Y + i * lda + i);
  hqr::tk::sub_dlarft(s, row - i, col - i, Y + i * lda + i, lda, TAU + i, T + i * ldt + i, ldt, base + g, 0);
  call.launched();
}

// tile_kernel.c:60-104
void tile_dtsqrt(const int row, const int col, const int block, double* A1, const int lda1, double* A2,
                 const int lda2, double* TAU, double* T, const int ldt, double* work) {
  (void)work;
  if (row <= 0 || col <= 0 || block <= 0) return;
  Call call("tile_dtsqrt");
  double* d1 = call.arg(A1, extent(lda1, col, col), true);
  double* d2 = call.arg(A2, extent(lda2, row, col), true);
  double* dtau = call.arg(TAU, col, true);
  double* dT = call.arg(T, extent(ldt, col, col), true);
  const size_t g = call.scratch((size_t)col * col);
  const size_t d = call.scratch((size_t)block * col), dd = call.scratch((size_t)block * col);
  double* base = call.bind();
  if (!base) return;
  A1 = call.view(A1, d1);
  A2 = call.view(A2, d2);
  TAU = call.view(TAU, dtau);
  T = call.view(T, dT);
  cudaStream_t s = call.stream();
  int i;
  for (i = 0; i < col - block; i += block) {
    hqr::tk::sub_dtsqr2(s, row, block, A1 + i + i * lda1, lda1, A2 + i * lda2, lda2, TAU + i);
    hqr::tk::sub_dlarft(s, row, block, A2 + i * lda2, lda2, TAU + i, T + i * ldt + i, ldt, base + g, 0);
    hqr::tk::sub_dssrfb(s, block, row, block, col - i - block, A2 + i * lda2, lda2, T + i + i * ldt, ldt,
                        A1 + i + (i + block) * lda1, lda1, A2 + (i + block) * lda2, lda2, base + d, base + dd,
                        nullptr, 0, 0);
  }
  if (col % block > 0) {
    i = block * (col / block);
    hqr::tk::sub_dtsqr2(s, row, col % block, A1 + i + i * lda1, lda1, A2 + i * lda2, lda2, TAU + i);
    hqr::tk::sub_dlarft(s, row, col % block, A2 + i * lda2, lda2, TAU + i, T + i * ldt + i, ldt, base + g, 0);
  } else {
    i = col - block;
    hqr::tk::sub_dtsqr2(s, row, block, A1 + i + i * lda1, lda1, A2 + i * lda2, lda2, TAU + i);
    hqr::tk::sub_dlarft(s, row, block, A2 + i * lda2, lda2, TAU + i, T + i * ldt + i, ldt, base + g, 0);
  }
  call.launched();
}

// tile_kernel.c:106-119
void tile_dlarfb(const int row, const int col, double* A, const int lda, const double* Y, const double* T,
                 const int ldt, double* work) {
  tile_sub_dlarfb(row, col, col, Y, lda, T, ldt, A, lda, work);
}

// tile_kernel.c:121-136
void tile_dssrfb(const int row, const int col, double* A1, double* A2, const int lda, const double* Y,
                 const double* T, const int ldt, double* work) {
  tile_sub_dssrfb(row, row, col, col, Y, lda, T, ldt, A1, lda, A2, lda, work);
}

// tile_kernel.c:368-437.  block < 2: the full lower T; 2 <= block < col: the
// coupling of the existing diagonal blocks; block >= col: T untouched.
void tile_dlarft(const int row, const int col, const int block, const double* Y, const int lda, const double* TAU,
                 double* T, const int ldt, double* work) {
  if (block < 2) {
    tile_sub_dlarft(row, col, Y, lda, TAU, T, ldt, work);
    return;
  }
  if (block >= col || row <= 0) return;
  Call call("tile_dlarft");
  double* dy = call.arg(Y, extent(lda, row, col), false);
  double* dT = call.arg(T, extent(ldt, col, col), true);
  const int ldg = (col / block) * block + block;
  const size_t g = call.scratch((size_t)col * ldg), t1 = call.scratch((size_t)col * block);
  double* base = call.bind();
  if (!base) return;
  hqr::tk::k_dlarft_block<<<1, hqr::kThreads, 0, call.stream()>>>(row, col, block, call.view(Y, dy), lda,
                                                                    call.view(T, dT), ldt, base + g, ldg,
                                                                    base + t1);
  call.launched();
}

// tile_kernel.c:439-476: A1 update of tile_dssrfb, W kept in upper_mat (ld row).
void tile_dssrfb_head(const int row, const int col, double* A1, double* A2, const int lda, const double* Y,
                      const double* T, const int ldt, double* upper_mat) {
  if (row <= 0 || col <= 0) return;
  Call call("tile_dssrfb_head");
  double* d1 = call.arg(A1, extent(lda, row, col), true);
  double* d2 = call.arg(A2, extent(lda, row, col), false);
  double* dy = call.arg(Y, extent(lda, row, col), false);
  double* dT = call.arg(T, extent(ldt, col, col), false);
  double* du = call.arg(upper_mat, (size_t)row * col, true);
  const size_t d = call.scratch((size_t)row * col), dd = call.scratch((size_t)col * col);
  double* base = call.bind();
  if (!base) return;
  hqr::tk::sub_dssrfb(call.stream(), row, row, col, col, call.view(Y, dy), lda, call.view(T, dT), ldt,
                      call.view(A1, d1), lda, call.view(A2, d2), lda, base + d, base + dd,
                      call.view(upper_mat, du), 1, 0);
  call.launched();
}

// tile_kernel.c:478-499: A2 -= Y W with W from tile_dssrfb_head.
void tile_dssrfb_tail(const int row, const int col, double* A2, const int lda, const double* Y, double* upper_mat) {
  if (row <= 0 || col <= 0) return;
  Call call("tile_dssrfb_tail");
  double* d2 = call.arg(A2, extent(lda, row, col), true);
  double* dy = call.arg(Y, extent(lda, row, col), false);
  double* du = call.arg(upper_mat, (size_t)row * col, false);
  if (!call.bind()) return;
  hqr::tk::sub_dssrfb(call.stream(), row, row, col, col, call.view(Y, dy), lda, nullptr, 0, nullptr, 0,
                      call.view(A2, d2), lda, nullptr, nullptr, call.view(upper_mat, du), 2, 0);
  call.launched();
}

// tile_kernel.c:501-601: tile_dlarfb with T read row-major (the transpose of
// the lower part of the column-major T).
void tile_return_dlarfb(const int row, const int col, double* A, const int lda, const double* Y, const double* T,
                        const int ldt, double* work) {
  (void)work;
  if (row <= 0 || col <= 0) return;
  Call call("tile_return_dlarfb");
  double* dy = call.arg(Y, extent(lda, row, col), false);
  double* dT = call.arg(T, extent(ldt, col, col), false);
  double* dA = call.arg(A, extent(lda, row, col), true);
  const size_t d = call.scratch((size_t)col * col), d2 = call.scratch((size_t)col * col);
  double* base = call.bind();
  if (!base) return;
  hqr::tk::sub_dlarfb(call.stream(), row, col, col, call.view(Y, dy), lda, call.view(T, dT), ldt, call.view(A, dA),
                      lda, base + d, base + d2, 1);
  call.launched();
}

// tile_kernel.c:603-650: tile_dssrfb with T read row-major.
void tile_return_dssrfb(const int row, const int col, double* A1, double* A2, const int lda, const double* Y,
                        const double* T, const int ldt, double* work) {
  (void)work;
  if (row <= 0 || col <= 0) return;
  Call call("tile_return_dssrfb");
  double* dy = call.arg(Y, extent(lda, row, col), false);
  double* dT = call.arg(T, extent(ldt, col, col), false);
  double* d1 = call.arg(A1, extent(lda, row, col), true);
  double* d2 = call.arg(A2, extent(lda, row, col), true);
  const size_t d = call.scratch((size_t)row * col), dd = call.scratch((size_t)col * col);
  double* base = call.bind();
  if (!base) return;
  hqr::tk::sub_dssrfb(call.stream(), row, row, col, col, call.view(Y, dy), lda, call.view(T, dT), ldt,
                      call.view(A1, d1), lda, call.view(A2, d2), lda, base + d, base + dd, nullptr, 0, 1);
  call.launched();
}

// Declared at tile_kernel.h:216 of the reference but never defined there:
// tile_sub_dlarft's T (built from a zeroed T), stored transposed in the upper
// triangle of T (ld ldt) as the tile_return_* kernels read it.
void tile_return_dlarft(const int row, const int col, const double* Y, const int lda, const double* TAU, double* T,
                        const int ldt, double* work) {
  (void)work;
  if (row <= 0 || col <= 0) return;
  Call call("tile_return_dlarft");
  double* dy = call.arg(Y, extent(lda, row, col), false);
  double* dtau = call.arg(TAU, col, false);
  double* dT = call.arg(T, extent(ldt, col, col), true);
  const size_t g = call.scratch((size_t)col * col), ts = call.scratch((size_t)col * col);
  double* base = call.bind();
  if (!base) return;
  cudaStream_t s = call.stream();
  if (cudaMemsetAsync(base + ts, 0, (size_t)col * col * sizeof(double), s) != cudaSuccess) {
    call.launched();
    return;
  }
  hqr::tk::sub_dlarft(s, row, col, call.view(Y, dy), lda, call.view(TAU, dtau), base + ts, col, base + g, 1);
  // copy the upper triangle (with the diagonal) into T
  T = call.view(T, dT);
  for (int c = 0; c < col; c++)
    if (cudaMemcpyAsync(T + (size_t)c * ldt, base + ts + (size_t)c * col, (size_t)(c + 1) * sizeof(double),
                        cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      break;
  call.launched();
}

}  // extern "C"
