// hqr_internal.h -- host-side interfaces shared by the library's translation
// units (not installed; the public C ABI is in include/).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "hqr_gpu.h"

namespace hqr {

// Geometry of one tiled matrix and the tile-kernel shape used on it.
struct Geometry {
  long M, N;       // rows / columns (multiples of NB)
  int NB, IB;      // tile order / requested inner block
  int MT, NT;      // tile rows / tile columns
  int steps;       // min(MT, NT)
  int w, CB, NC;   // inner block width, column-block width, column blocks per tile
  size_t smem_bytes;
};

// smem_limit: bytes of dynamic shared memory the executor may use (0: one CTA
// per SM); the update tasks' column block narrows to fit.
int make_geometry(long M, long N, int NB, int IB, Geometry* g, size_t smem_limit = 0);

// Remember the text of a failed CUDA call (reported by hqr_last_cuda_error)
// and return HQR_ERR_CUDA.
int record_cuda_error(cudaError_t e, const char* where);
// Report a drop-in entry point's status the way the error mode says (print
// and exit, or print and remember for hqr_last_error); returns rc.
int report_error(const char* fn, int rc);

// Column-major (M x N, ld) <-> tile layout padded to whole tiles (hqr_util.cu).
void colmajor_to_tiles_padded(const double* dIn, long ld, long M, long N, int NB, double* dT, cudaStream_t s);
void tiles_to_colmajor_padded(const double* dT, long ld, long M, long N, int NB, double* dOut, cudaStream_t s);

// Least-squares helpers (hqr_lstsq.cu).  Right-hand sides: column-major
// M x nrhs; C: tile layout with MT = M / NB tile rows and CT tile columns.
void pack_rhs(const double* dB, long ldb, int nrhs, double* dC, long M, int NB, int CT, cudaStream_t s);
void update_x(const double* dC, long M, int NB, long N, int nrhs, double* dX, long ldx, bool accumulate,
              cudaStream_t s);
int residual(const double* dA, long M, long N, int NB, const double* dX, long ldx, const double* dB,
             long ldb, double* dR, long ldr, int nrhs, cudaStream_t s);
void col_norm2(const double* dR, long M, long ldr, int nrhs, double* dOut, cudaStream_t s);
// Back substitution R Y = C(1:N, :) in place (R: upper triangle of the
// factored A's first N / NB tile rows).
int trsm_tiles(const double* dRA, long M, long N, int NB, double* dC, int nrhs, cudaStream_t s);
// Forward substitution R^T Y = C(1:N, :) in place.
int trsmt_tiles(const double* dRA, long M, long N, int NB, double* dC, int nrhs, cudaStream_t s);
// pack_rhs with rows nrows.. of the tile layout zero.
void pack_rhs_rows(const double* dB, long ldb, int nrhs, long nrows, double* dC, long M, int NB, int CT,
                   cudaStream_t s);
void sub_colmajor(double* dF, long ldf, const double* dR, long ldr, long M, int nrhs, cudaStream_t s);
// R (column-major) += the first nrhs columns of D (tile layout).
void add_unpack(double* dR, long ldr, const double* dD, long M, int NB, int nrhs, cudaStream_t s);
// Tile rows [ti0, ti1) of MT x CT tile grids: D <- C, or C -= D (sub).
void tile_rows(double* dC, double* dD, long M, int NB, int CT, int ti0, int ti1, bool sub, cudaStream_t s);
// Tile-row slices of at_times for about four blocks per SM.
int atr_slices(long M, long N, int NB, int nrhs);
// G (column-major N x nrhs) = alpha A^T R (R column-major M x nrhs) in FP64,
// over S slices of tile rows summed in a fixed order (dP: S N nrhs doubles).
int at_times(const double* dA, long M, long N, int NB, const double* dR, long ldr, int nrhs, double alpha,
             double* dG, long ldg, double* dP, int S, cudaStream_t s);

// Scheduler workspace (dependency counters, queues, control words, stats).
struct DagWorkspace {
  int* cnt = nullptr;
  int* flag = nullptr;   // per panel block: its trailing update is done (factorization)
  int* qhi = nullptr;
  int* qlo = nullptr;
  unsigned* ctl = nullptr;
  unsigned long long* stats = nullptr;
  size_t cap_ids = 0;
};

int dag_workspace_reserve(DagWorkspace* ws, size_t n_ids);
void dag_workspace_free(DagWorkspace* ws);

// Workspace of the split-precision updates (null slices: FP64 updates).
struct OzWorkspace {
  uint8_t* slices = nullptr;   // sliced V^T, T^T, V, T of every panel tile
  int* sexp = nullptr;         // their row exponents
  int groups = 8;              // t-groups of the updates: 8 (FP64-level) or 4 (reduced)
  int fp32_panels = 0;         // 1: the factorization's panel blocks compute in FP32
};
// Bytes of the split-precision workspace for a geometry (NB = 128).
size_t oz_slice_bytes(const Geometry& g);
size_t oz_exp_bytes(const Geometry& g);
size_t oz_exp_bytes_per_panel(int NB);   // row exponents of one panel tile's operands
size_t oz_panel_bytes();   // prepared operands of one panel tile
bool oz_supported(const Geometry& g);
// Inner block width of the FP64 panels for the split path (see hqr_dag.cu).
int narrow_panels(Geometry* g);

// Domain tree of a plan: domains of S tiles (0: the flat tree) and the
// merges' storage, compact per (step i, domain d): T2 tile (i*dmax + d), TAU2
// (i*dmax + d)*NB, and for split precision their prepared operands.
struct TreeWorkspace {
  int S = 0;
  double* T2 = nullptr;
  double* TAU2 = nullptr;
  uint8_t* slices2 = nullptr;
  int* sexp2 = nullptr;
};
// Number of merge slots of a tree with domains of S tiles (steps * dmax).
size_t tree_slots(const Geometry& g, int S);

// Enqueue a factorization DAG on `stream` (no synchronisation).
int launch_factor(const Geometry& g, DagWorkspace* ws, double* dA, double* dT, double* dTAU,
                  long long timeout_ns, cudaStream_t stream, const OzWorkspace* oz = nullptr,
                  const TreeWorkspace* tw = nullptr);
// C <- Q^T C for a factorization with a domain tree, from the T factors (or
// split slices) that factorization left in dT / tw / oz.
int launch_apply_qt_tree(const Geometry& g, DagWorkspace* ws, const double* dA, double* dT,
                         const double* dTAU, double* dC, int CT, long long timeout_ns, cudaStream_t stream,
                         const OzWorkspace* oz, const TreeWorkspace* tw);
// Enqueue C <- Q^T C (C has CT tile columns, same MT/NB as A); the panel
// tasks rebuild T from V/TAU (FP64: diagonal blocks; split: full T + slices).
// ccols > 0: only C's first ccols columns hold data (the rest are zero and
// stay so); the updates of column blocks beyond them are skipped.
int launch_apply_qt(const Geometry& g, DagWorkspace* ws, const double* dA, double* dT,
                    const double* dTAU, double* dC, int CT, bool rebuild_t, long long timeout_ns,
                    cudaStream_t stream, const OzWorkspace* oz = nullptr, long long ccols = 0);
// Q = H_0 H_1 ... H_{steps-1} dQ for dQ = I (square matrices): backward
// accumulation, skipping the tile columns that are still unit vectors.
// rebuild_t false: the T factors / prepared operands of the factorization.
int launch_build_q(const Geometry& g, DagWorkspace* ws, const double* dA, double* dT, const double* dTAU,
                   double* dQ, bool rebuild_t, long long timeout_ns, cudaStream_t stream,
                   const OzWorkspace* oz = nullptr);
// C <- Q C (CT tile columns, same MT/NB as A): H applied in backward order;
// rebuild_t false: the T factors / prepared operands (of H) given.
int launch_apply_q(const Geometry& g, DagWorkspace* ws, const double* dA, double* dT, const double* dTAU,
                   double* dC, int CT, bool rebuild_t, long long timeout_ns, cudaStream_t stream,
                   const OzWorkspace* oz = nullptr, long long ccols = 0);
// Batches of independent FP64 factorizations in one persistent launch.
// Descriptors (mat_desc_bytes() each) are written to host memory by
// batch_describe and must be on the device (d_desc) for launch_batch.
size_t mat_desc_bytes();
// apply: C <- Q^T C on the first nrhs columns of each C (else the factorization).
long long batch_ids(bool apply, const Geometry& g, int nrhs);
// order (or null): the matrices in the order of the table (and of the first
// tasks queued: the init and seed kernels run one block per table entry).
int batch_describe(bool apply, int count, const Geometry* gs, const int* order, double* const* A,
                   double* const* T, double* const* TAU, double* const* C, int nrhs, void* desc, int* n_ids,
                   int* n_tasks);
// Dynamic shared memory per executor CTA that lets two CTAs share an SM.
size_t batch_two_cta_smem();
// ctas_per_sm: executor CTAs per SM (0: as many as fit, at most 2).
int launch_batch(bool apply, int count, const void* d_desc, int n_ids, int n_tasks, size_t smem,
                 int ctas_per_sm, DagWorkspace* ws, long long timeout_ns, cudaStream_t stream);
// Scratch supplied by the caller instead of a DagWorkspace (no allocation).
struct ExternalScratch {
  double* T;
  int* cnt;
  int* qhi;
  int* qlo;
  unsigned* ctl;                 // control words, zeroed by the caller
  unsigned long long* stats;     // 10 counters, zeroed by the caller
};
constexpr int kExternalCtlBytes = 8 * 4;
constexpr int kExternalStatsBytes = 14 * 8;
// Number of task ids of the factorization DAG (size of cnt / qhi / qlo).
size_t factor_task_ids(const Geometry& g);
// Enqueue the factorization DAG on caller-supplied scratch.
int launch_factor_external(const Geometry& g, const ExternalScratch& x, double* dA, double* dTAU,
                           long long timeout_ns, cudaStream_t stream);
// Synchronise `stream` and read the error word of caller-supplied scratch.
int external_status(const ExternalScratch& x, cudaStream_t stream);
// Read and clear the scheduler's error word (synchronises `stream`).
int dag_status(DagWorkspace* ws, cudaStream_t stream);
int dag_stats(DagWorkspace* ws, unsigned long long out[14], cudaStream_t stream);
int dag_sm_count();

// Utility kernels (hqr_util.cu)
void fill_uniform(double* dA, long M, long N, int NB, uint64_t seed, cudaStream_t s);
void make_identity(double* dQ, long M, long N, int NB, bool zero_first, cudaStream_t s);
// In-place transpose of a square N x N tile-layout matrix (NB a multiple of 32).
void transpose_tiles(double* dQ, long N, int NB, cudaStream_t s);
// Host <-> device copies of n doubles for the drop-in calls.  A host array
// that is page-locked and mapped (cudaHostAlloc, cudaHostRegister) is moved
// by SM loads / stores through its device mapping: on this part the copy
// engines' rate to host memory drops at times to a tenth, the SMs' does not.
// Pageable host memory goes through cudaMemcpyAsync.
cudaError_t copy_host_to_device(double* d, const double* h, size_t n, cudaStream_t s);
cudaError_t copy_device_to_host(double* h, const double* d, size_t n, cudaStream_t s);
void zero_reflectors(double* dA, long M, long N, int NB, cudaStream_t s);
void dgemm_tn_tiles(const double* dA, const double* dB, double* dC, long M, long N, int NB,
                    cudaStream_t s);
// sum of squares of (X - alpha*I - Y) over the tile array (Y may be null);
// result written to *d_out (device double).
void frob_diff(const double* dX, const double* dY, double alpha_identity, long M, long N, int NB,
               double* d_out, cudaStream_t s);
void tiles_to_colmajor(const double* dT, double* dOut, long M, long N, int NB, cudaStream_t s);
void colmajor_to_tiles(const double* dIn, double* dT, long M, long N, int NB, cudaStream_t s);
void max_col_abs_sum(const double* dColMajor, long M, long N, double* d_out, cudaStream_t s);
double measure_fp64_peak_tflops(cudaStream_t s);
double measure_fp64_mma_peak_tflops(int shape, cudaStream_t s);

}  // namespace hqr
