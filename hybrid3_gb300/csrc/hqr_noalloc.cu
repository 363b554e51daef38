// hqr_noalloc.cu -- a factorization entry point that allocates no memory.
//
// hqr_geqrf_noalloc runs the same tile DAG as hqr_geqrf, but the scratch that
// hqr_geqrf obtains from cudaMalloc (the T factors of every panel tile, the
// DAG's dependency counters and ready queues, the scheduler's control words)
// lives in one fixed-size array in device global memory, reserved when the
// library's device code is loaded.  It exists for callers that may not call
// cudaMalloc: processes whose device memory is entirely owned by their own
// pool allocator, and latency-bound paths that cannot afford the device-wide
// synchronisation an allocation can cause.  They pass device pointers to A and
// TAU and nothing else.  Each call ends by synchronising its stream and
// reading the scheduler's error word.
//
// Limits and sharing:
//   * the array holds kNoAllocScratchBytes (64 MiB) on every GPU that loads
//     the library, until the process exits;
//   * a shape is accepted when its T factors (M*N doubles) plus scheduler
//     tables fit: about n <= 2800 for a square matrix (2048 x 2048 with
//     NB = 256 uses 32 MiB);
//   * every call, on every stream, uses the same array: calls that overlap on
//     the GPU race and corrupt each other -- serialise them;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) and caches it; make that first call before any
//     stream capture begins;
//   * the scheduler's wait limit is fixed at 20 s here (hqr_set_timeout_ms
//     does not apply).
#include <cstdio>
#include <mutex>

#include "hqr_internal.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;
constexpr int kMaxDevices = 64;

// The scratch.  In host code this name only stands for the symbol; it is not
// a device address.  The address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_addr[kMaxDevices] = {};

size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

// Device address of the scratch on the current device, looked up on the first
// call made with that device current and cached.
int noalloc_scratch(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return hqr::record_cuda_error(e, "hqr_geqrf_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return HQR_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return hqr::record_cuda_error(e, "hqr_geqrf_noalloc: cudaGetSymbolAddress");
    if (!p) return HQR_ERR_CUDA;
    g_noalloc_addr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_noalloc_addr[dev]);
  return HQR_OK;
}

}  // namespace

extern "C" int hqr_geqrf_noalloc(long M, long N, int NB, int IB, double* dA, double* dTAU,
                                 void* stream) {
  if (!dA || !dTAU) return HQR_ERR_INVALID;
  hqr::Geometry g;
  int rc = hqr::make_geometry(M, N, NB, IB, &g);
  if (rc != HQR_OK) return rc;

  // carve the scratch: T factors | counters | two queues | control | stats
  const size_t n_ids = hqr::factor_task_ids(g);
  const size_t b_t = round256((size_t)M * (size_t)N * sizeof(double));
  const size_t b_ids = round256(n_ids * sizeof(int));
  const size_t b_ctl = round256(hqr::kExternalCtlBytes);
  const size_t b_stats = round256(hqr::kExternalStatsBytes);
  const size_t need = b_t + 3 * b_ids + b_ctl + b_stats;
  if (need > kNoAllocScratchBytes) {
    fprintf(stderr,
            "hqr_geqrf_noalloc: a %ld x %ld matrix with NB = %d needs %zu bytes of scratch; "
            "the fixed scratch holds %zu bytes\n",
            M, N, NB, need, kNoAllocScratchBytes);
    return HQR_ERR_UNSUPPORTED;
  }
  unsigned char* base = nullptr;
  rc = noalloc_scratch(&base);
  if (rc != HQR_OK) return rc;
  hqr::ExternalScratch x;
  size_t off = 0;
  x.T = reinterpret_cast<double*>(base + off);
  off += b_t;
  x.cnt = reinterpret_cast<int*>(base + off);
  off += b_ids;
  x.qhi = reinterpret_cast<int*>(base + off);
  off += b_ids;
  x.qlo = reinterpret_cast<int*>(base + off);
  off += b_ids;
  x.ctl = reinterpret_cast<unsigned*>(base + off);
  off += b_ctl;
  x.stats = reinterpret_cast<unsigned long long*>(base + off);

  cudaStream_t s = (cudaStream_t)stream;
  // The array keeps the previous call's contents.  The control words and the
  // statistics must start at zero; the counters and queues are written by the
  // DAG's init kernel, and every T block is written by its panel task before
  // any update reads it.
  cudaError_t e = cudaMemsetAsync(x.ctl, 0, b_ctl, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(x.stats, 0, b_stats, s);
  if (e != cudaSuccess) return hqr::record_cuda_error(e, "hqr_geqrf_noalloc: scratch reset");
  rc = hqr::launch_factor_external(g, x, dA, dTAU, 20000LL * 1000000LL, s);
  if (rc != HQR_OK) return rc;
  return hqr::external_status(x, s);
}
