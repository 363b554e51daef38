// hqr_dag.cu -- host side of the device DAG: geometry, workspace and launches
// of the persistent executor for the factorization and the Q^T application.
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "hqr_dag.cuh"
#include "hqr_internal.h"

namespace hqr {

int make_geometry(long M, long N, int NB, int IB, Geometry* g, size_t smem_limit) {
  if (NB < 16 || NB > kMaxNB || NB % 16 != 0) return HQR_ERR_UNSUPPORTED;
  if (M <= 0 || N <= 0 || M % NB != 0 || N % NB != 0) return HQR_ERR_INVALID;
  if (IB <= 0 || IB > NB) return HQR_ERR_INVALID;
  g->M = M;
  g->N = N;
  g->NB = NB;
  g->IB = IB;
  g->MT = (int)(M / NB);
  g->NT = (int)(N / NB);
  g->steps = std::min(g->MT, g->NT);
  // inner block: the largest divisor of NB that is <= min(IB, 32) and a multiple of 8
  int w = std::min(IB, kMaxW);
  w -= w % 8;
  while (w > 8 && NB % w != 0) w -= 8;
  if (w < 8) w = 8;
  g->w = w;
  // column block of the update tasks: the widest multiple of 8 dividing NB,
  // at most 64 and at most NB*CB*8 <= 64 KiB, whose shared-memory plan fits
  const size_t smem_cap = smem_limit ? smem_limit : 227 * 1024 - 256;   // room for static shared memory
  int cb = (8192 / NB) > 64 ? 64 : 8192 / NB;
  if (cb > NB) cb = NB;
  cb -= cb % 8;
  for (; cb >= 8; cb -= 8) {
    if (NB % cb != 0) continue;
    TileShape sh{NB, w, cb, NB >= 512 ? 64 : kRC};
    if ((size_t)SmemPlan::make(sh).total * sizeof(double) <= smem_cap) break;
  }
  if (cb < 8) return HQR_ERR_UNSUPPORTED;
  g->CB = cb;
  g->NC = NB / cb;
  TileShape sh{NB, w, cb, NB >= 512 ? 64 : kRC};
  SmemPlan sp = SmemPlan::make(sh);
  g->smem_bytes = (size_t)sp.total * sizeof(double);
  if (g->smem_bytes > smem_cap) return HQR_ERR_UNSUPPORTED;
  if ((long long)g->steps * g->MT * (g->NB / g->w + 1) + (long long)g->steps * g->NT * g->MT * g->NC >
      0x3fffffffLL)
    return HQR_ERR_UNSUPPORTED;
  return HQR_OK;
}

static TileShape shape_of(const Geometry& g) {
  return TileShape{g.NB, g.w, g.CB, g.NB >= 512 ? 64 : kRC};
}

int dag_workspace_reserve(DagWorkspace* ws, size_t n_ids) {
  if (ws->cap_ids >= n_ids && ws->ctl) return HQR_OK;
  dag_workspace_free(ws);
  if (cudaMalloc(&ws->cnt, n_ids * sizeof(int)) != cudaSuccess) return HQR_ERR_NOMEM;
  if (cudaMalloc(&ws->flag, n_ids * sizeof(int)) != cudaSuccess) return HQR_ERR_NOMEM;
  if (cudaMalloc(&ws->qhi, n_ids * sizeof(int)) != cudaSuccess) return HQR_ERR_NOMEM;
  if (cudaMalloc(&ws->qlo, n_ids * sizeof(int)) != cudaSuccess) return HQR_ERR_NOMEM;
  if (cudaMalloc(&ws->ctl, kCtlWords * sizeof(unsigned)) != cudaSuccess) return HQR_ERR_NOMEM;
  if (cudaMalloc(&ws->stats, 2 * kNumStats * sizeof(unsigned long long)) != cudaSuccess)
    return HQR_ERR_NOMEM;
  if (cudaMemset(ws->ctl, 0, kCtlWords * sizeof(unsigned)) != cudaSuccess) return HQR_ERR_CUDA;
  ws->cap_ids = n_ids;
  return HQR_OK;
}

void dag_workspace_free(DagWorkspace* ws) {
  if (ws->cnt) cudaFree(ws->cnt);
  if (ws->flag) cudaFree(ws->flag);
  if (ws->qhi) cudaFree(ws->qhi);
  if (ws->qlo) cudaFree(ws->qlo);
  if (ws->ctl) cudaFree(ws->ctl);
  if (ws->stats) cudaFree(ws->stats);
  *ws = DagWorkspace{};
}

// Per-device caches: cudaFuncSetAttribute applies to the current device only,
// and the SM count is a property of the device, so both are kept per device
// ordinal (devices beyond kCacheDevices are simply not cached).
constexpr int kCacheDevices = 64;
static int current_device() {
  int dev = 0;
  return cudaGetDevice(&dev) == cudaSuccess ? dev : -1;
}

int dag_sm_count() {
  static int n[kCacheDevices] = {};
  const int dev = current_device();
  const bool cached = dev >= 0 && dev < kCacheDevices;
  if (cached && n[dev] > 0) return n[dev];
  int v = 0;
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev < 0 ? 0 : dev);
  if (v <= 0) v = 1;
  if (cached) n[dev] = v;
  return v;
}

// The largest dynamic shared memory a kernel has been opted in to, per device.
struct SmemOptIn {
  std::mutex mu;
  size_t bytes[kCacheDevices] = {};
};
// Opt `kernel` in to smem bytes of dynamic shared memory on the current device
// (once per device and size); extra(): further attribute calls made with it.
template <class Kernel, class Extra>
static cudaError_t opt_in(SmemOptIn& o, Kernel kernel, size_t smem, Extra extra) {
  const int dev = current_device();
  std::lock_guard<std::mutex> lk(o.mu);
  if (dev >= 0 && dev < kCacheDevices && smem <= o.bytes[dev]) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = extra();
  if (e == cudaSuccess && dev >= 0 && dev < kCacheDevices) o.bytes[dev] = smem;
  return e;
}
template <class Kernel>
static cudaError_t opt_in(SmemOptIn& o, Kernel kernel, size_t smem) {
  return opt_in(o, kernel, smem, [] { return cudaSuccess; });
}

static size_t dag_smem_bytes(const Geometry& g, bool oz) {
  size_t b = g.smem_bytes;
  if (oz) b = std::max(b, (size_t)oz::kSmemBytes);
  return b;
}

template <bool OZ, int G = 8, bool P32 = false>
static int launch_exec(const DagParams& p, const Geometry& g, cudaStream_t stream) {
  static SmemOptIn opted;
  const size_t smem = dag_smem_bytes(g, OZ);
  {
    const cudaError_t e = opt_in(opted, dag_exec_kernel<OZ, false, G, P32>, smem);
    if (e != cudaSuccess) return record_cuda_error(e, "cudaFuncSetAttribute(dag_exec_kernel)");
  }
  const int grid = std::min(dag_sm_count(), std::max(1, p.n_tasks));
  dag_exec_kernel<OZ, false, G, P32><<<grid, kThreads, smem, stream>>>(p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return record_cuda_error(e, "dag_exec_kernel launch");
  return HQR_OK;
}

static int run_dag(DagParams& p, DagWorkspace* ws, const Geometry& g, cudaStream_t stream) {
  p.sh = shape_of(g);
  p.sp = SmemPlan::make(p.sh);
  p.n_ids = id_end(p);
  int rc = dag_workspace_reserve(ws, (size_t)p.n_ids);
  if (rc != HQR_OK) return rc;
  p.cnt = ws->cnt;
  p.tsflag = ws->flag;
  p.qhi = ws->qhi;
  p.qlo = ws->qlo;
  p.ctl = ws->ctl;
  p.stats = ws->stats;
  // control words: queue heads/tails and the done counter start at zero; the
  // error word is kept (cleared by dag_status) so a failure is never lost.
  cudaError_t e0 = cudaMemsetAsync(ws->ctl, 0, kErr * sizeof(unsigned), stream);
  if (e0 == cudaSuccess)
    e0 = cudaMemsetAsync(ws->stats, 0, 2 * kNumStats * sizeof(unsigned long long), stream);
  if (e0 != cudaSuccess) return record_cuda_error(e0, "DAG workspace reset");
  const int blocks = (p.n_ids + 255) / 256;
  dag_init_kernel<<<blocks, 256, 0, stream>>>(p);
  dag_seed_kernel<<<blocks, 256, 0, stream>>>(p);
  if (!p.oz) return launch_exec<false>(p, g, stream);
  if (p.oz_groups == 8) return launch_exec<true, 8>(p, g, stream);
  return p.oz_p32 ? launch_exec<true, 4, true>(p, g, stream) : launch_exec<true, 4>(p, g, stream);
}

// Update tiles left in a step below which the factorization's panel blocks
// run in phases (DagParams::ts_split).
constexpr long long kPhasedWork = 6000;

// 64-column chunks per split update task, run one after the other: two (a
// whole 128-column tile) halve the number of update tasks and with them the
// scheduling round trips (a queue claim and the dependents' releases, about
// 6 us per task), at the price of half the tasks per step.
constexpr int kOzChunksPerTask = 2;
static void set_oz(DagParams& p, const Geometry& g, const OzWorkspace* oz) {
  if (oz && oz->slices) {
    p.oz = 1;
    p.oz_groups = oz->groups;
    p.oz_p32 = oz->fp32_panels;
    p.oz_cpt = kOzChunksPerTask;
    p.NC = g.NB / oz::kN / p.oz_cpt;
    p.slices = oz->slices;
    p.sexp = oz->sexp;
  } else {
    p.oz = 0;
    p.NC = g.NC;
  }
}

// Domains and merge storage of a domain tree (tw null or tw->S == 0: flat).
static void set_tree(DagParams& p, const Geometry& g, const TreeWorkspace* tw) {
  if (!tw || tw->S <= 0 || tw->S >= g.MT) {
    p.tree = 0;
    p.dmax = 0;
    return;
  }
  p.tree = tw->S;
  p.dmax = (g.MT + tw->S - 1) / tw->S;
  p.T2 = tw->T2;
  p.TAU2 = tw->TAU2;
  p.slices2 = tw->slices2;
  p.sexp2 = tw->sexp2;
}
static long long merges_of_step(const DagParams& p, int i) { return n_domains(p, i) - 1; }

int launch_factor(const Geometry& g, DagWorkspace* ws, double* dA, double* dT, double* dTAU,
                  long long timeout_ns, cudaStream_t stream, const OzWorkspace* ozw,
                  const TreeWorkspace* tw) {
  DagParams p{};
  p.mode = kModeFactor;
  p.MT = g.MT;
  p.NT = g.NT;
  p.CT = g.NT;
  p.steps = g.steps;
  p.J = g.NT;
  p.A = dA;
  p.T = dT;
  p.TAU = dTAU;
  p.C = dA;
  p.timeout_ns = timeout_ns;
  set_oz(p, g, ozw);
  p.prep = p.oz;
  p.nblk = g.NB / g.w;
  set_tree(p, g, tw);
  // split precision, flat tree: panel blocks release their panel dependents
  // in phases (the first trailing column block is then w wide, which changes
  // the rounding of the FP64 panels' trailing sums, so FP64 plans keep the
  // whole-block releases and their results)
  p.ts_split = (p.tree == 0 && p.oz) ? 1 : 0;
  // only in the steps whose panel chain, not their update work, sets the
  // pace: few update tiles left ((NT - i - 1) (MT - i - 1) at most
  // kPhasedWork); before them the phases' waits and narrower first column
  // block cost more than the shorter chain gains
  p.ts_split_from = 0;
  while (p.ts_split_from < g.steps &&
         (long long)(g.NT - p.ts_split_from - 1) * (g.MT - p.ts_split_from - 1) > kPhasedWork)
    p.ts_split_from++;
  // tasks: per step i, nblk inner blocks of each of the MT-i panel tiles [+ one
  // OZPREP per panel tile] + NC*(NT-1-i)*(MT-i) updates; a tree adds per merge
  // nblk blocks [+ one OZPREP] + NC*(NT-1-i) merge updates
  long long n = 0;
  for (int i = 0; i < g.steps; i++) {
    const long long m = merges_of_step(p, i);
    n += (long long)(g.MT - i) * (p.nblk + (p.prep ? 1 : 0)) + (long long)p.NC * (g.NT - 1 - i) * (g.MT - i);
    n += m * (p.nblk + (p.prep ? 1 : 0)) + m * p.NC * (g.NT - 1 - i);
  }
  p.n_tasks = (int)n;
  return run_dag(p, ws, g, stream);
}

int launch_apply_qt(const Geometry& g, DagWorkspace* ws, const double* dA, double* dT,
                    const double* dTAU, double* dC, int CT, bool rebuild_t, long long timeout_ns,
                    cudaStream_t stream, const OzWorkspace* ozw, long long ccols) {
  if (CT <= 0) return HQR_ERR_INVALID;
  DagParams p{};
  p.mode = kModeApplyQt;
  p.c_cols = ccols;
  p.MT = g.MT;
  p.NT = g.NT;
  p.CT = CT;
  p.steps = g.steps;
  p.J = CT;
  p.A = const_cast<double*>(dA);
  p.T = dT;
  p.TAU = const_cast<double*>(dTAU);
  p.C = dC;
  p.timeout_ns = timeout_ns;
  set_oz(p, g, ozw);
  p.prep = 0;
  p.nblk = 1;
  // rebuild_t: panel tasks rebuild each panel tile's T (FP64: its diagonal
  // blocks) or prepared operands (split) from V and TAU; else the updates use
  // those the factorization left in dT / the slice store
  p.skip_panels = rebuild_t ? 0 : 1;
  long long n = 0;
  for (int i = 0; i < g.steps; i++) n += (rebuild_t ? (g.MT - i) : 0) + (long long)p.NC * CT * (g.MT - i);
  p.n_tasks = (int)n;
  return run_dag(p, ws, g, stream);
}

int launch_apply_qt_tree(const Geometry& g, DagWorkspace* ws, const double* dA, double* dT,
                         const double* dTAU, double* dC, int CT, long long timeout_ns, cudaStream_t stream,
                         const OzWorkspace* ozw, const TreeWorkspace* tw) {
  if (CT <= 0 || !tw || tw->S <= 0) return HQR_ERR_INVALID;
  DagParams p{};
  p.mode = kModeApplyQt;
  p.MT = g.MT;
  p.NT = g.NT;
  p.CT = CT;
  p.steps = g.steps;
  p.J = CT;
  p.A = const_cast<double*>(dA);
  p.T = dT;
  p.TAU = const_cast<double*>(dTAU);
  p.C = dC;
  p.timeout_ns = timeout_ns;
  set_oz(p, g, ozw);
  p.prep = 0;
  p.nblk = 1;
  p.skip_panels = 1;   // the T factors / slices of the factorization on this plan
  set_tree(p, g, tw);
  long long n = 0;
  for (int i = 0; i < g.steps; i++) n += (long long)p.NC * CT * ((g.MT - i) + merges_of_step(p, i));
  p.n_tasks = (int)n;
  return run_dag(p, ws, g, stream);
}

int launch_build_q(const Geometry& g, DagWorkspace* ws, const double* dA, double* dT, const double* dTAU,
                   double* dQ, bool rebuild_t, long long timeout_ns, cudaStream_t stream, const OzWorkspace* ozw) {
  if (g.M != g.N) return HQR_ERR_INVALID;
  DagParams p{};
  p.mode = kModeBuildQ;
  p.MT = g.MT;
  p.NT = g.NT;
  p.CT = g.NT;
  p.steps = g.steps;
  p.J = g.NT;
  p.A = const_cast<double*>(dA);
  p.T = dT;
  p.TAU = const_cast<double*>(dTAU);
  p.C = dQ;
  p.timeout_ns = timeout_ns;
  set_oz(p, g, ozw);
  p.prep = 0;
  p.nblk = 1;
  p.skip_panels = rebuild_t ? 0 : 1;   // as in launch_apply_qt (split: T from its own slot)
  // per step i: MT - i panel tasks (when rebuilding) and NC (NT - i) (MT - i) updates
  long long n = 0;
  for (int i = 0; i < g.steps; i++)
    n += (rebuild_t ? (g.MT - i) : 0) + (long long)p.NC * (g.NT - i) * (g.MT - i);
  p.n_tasks = (int)n;
  return run_dag(p, ws, g, stream);
}

int launch_apply_q(const Geometry& g, DagWorkspace* ws, const double* dA, double* dT, const double* dTAU,
                   double* dC, int CT, bool rebuild_t, long long timeout_ns, cudaStream_t stream,
                   const OzWorkspace* ozw, long long ccols) {
  if (CT <= 0) return HQR_ERR_INVALID;
  DagParams p{};
  p.mode = kModeApplyQ;
  p.c_cols = ccols;
  p.MT = g.MT;
  p.NT = g.NT;
  p.CT = CT;
  p.steps = g.steps;
  p.J = CT;
  p.A = const_cast<double*>(dA);
  p.T = dT;
  p.TAU = const_cast<double*>(dTAU);
  p.C = dC;
  p.timeout_ns = timeout_ns;
  set_oz(p, g, ozw);
  p.prep = 0;
  p.nblk = 1;
  p.skip_panels = rebuild_t ? 0 : 1;
  long long n = 0;
  for (int i = 0; i < g.steps; i++) n += (rebuild_t ? (g.MT - i) : 0) + (long long)p.NC * CT * (g.MT - i);
  p.n_tasks = (int)n;
  return run_dag(p, ws, g, stream);
}

// --- batches of independent matrices (FP64) ---------------------------------------
size_t mat_desc_bytes() { return sizeof(MatDesc); }

// The per-matrix fields of a batch launch (factorization, or C <- Q^T C with
// the T factors the factorization left), plus that matrix's id / task counts.
// C <- Q^T C covers the first nrhs columns of C: ceil(nrhs / NB) tile
// columns; fewer than NB right-hand sides take the narrowest column blocks
// (a multiple of 8 dividing NB, at most the factorization's) that hold them.
static DagParams batch_matrix_params(bool apply, const Geometry& g, int nrhs) {
  DagParams p{};
  p.mode = apply ? kModeApplyQt : kModeFactor;
  p.MT = g.MT;
  p.NT = g.NT;
  p.NC = g.NC;
  p.steps = g.steps;
  p.CT = g.NT;
  p.nblk = g.NB / g.w;
  p.sh = shape_of(g);
  if (apply) {
    p.skip_panels = 1;
    p.nblk = 1;
    p.CT = (nrhs + g.NB - 1) / g.NB;
    if (nrhs < g.NB) {
      int cb = (nrhs + 7) / 8 * 8;
      while (cb < g.CB && g.NB % cb != 0) cb += 8;
      if (cb > g.CB) cb = g.CB;
      p.sh.CB = cb;
      p.NC = (nrhs + cb - 1) / cb;
    }
  }
  p.J = p.CT;
  p.sp = SmemPlan::make(p.sh);
  return p;
}
static long long batch_matrix_tasks(bool apply, const DagParams& p) {
  long long n = 0;
  for (int i = 0; i < p.steps; i++) {
    if (apply)
      n += (long long)p.NC * p.CT * (p.MT - i);
    else
      n += (long long)(p.MT - i) * p.nblk + (long long)p.NC * (p.NT - 1 - i) * (p.MT - i);
  }
  return n;
}

long long batch_ids(bool apply, const Geometry& g, int nrhs) {
  return id_end(batch_matrix_params(apply, g, nrhs));
}

int batch_describe(bool apply, int count, const Geometry* gs, const int* order, double* const* A,
                   double* const* T, double* const* TAU, double* const* C, int nrhs, void* desc, int* n_ids,
                   int* n_tasks) {
  MatDesc* d = static_cast<MatDesc*>(desc);
  long long ids = 0, tasks = 0;
  for (int i = 0; i < count; i++) {
    const int b = order ? order[i] : i;
    const DagParams p = batch_matrix_params(apply, gs[b], nrhs);
    MatDesc m{};
    m.MT = p.MT;
    m.NT = p.NT;
    m.CT = p.CT;
    m.NC = p.NC;
    m.steps = p.steps;
    m.J = p.J;
    m.nblk = p.nblk;
    m.sh = p.sh;
    m.sp = p.sp;
    m.A = A[b];
    m.T = T[b];
    m.TAU = TAU[b];
    m.C = apply ? C[b] : A[b];
    m.id_base = (int)ids;
    ids += id_end(p);
    tasks += batch_matrix_tasks(apply, p);
    if (ids > 0x3fffffffLL) return HQR_ERR_UNSUPPORTED;
    m.id_end = (int)ids;
    d[i] = m;
  }
  *n_ids = (int)ids;
  *n_tasks = (int)tasks;
  return HQR_OK;
}

size_t batch_two_cta_smem() {
  static size_t v = 0;
  if (v == 0) {
    int dev = 0, per_sm = 0;
    cudaFuncAttributes fa{};
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaFuncGetAttributes(&fa, dag_exec_kernel<false, true>);
    // per CTA: the dynamic part, the kernel's static part and 1 KiB the system reserves
    const long long b = (long long)per_sm / 2 - (long long)fa.sharedSizeBytes - 1024;
    v = b > 0 ? (size_t)b : 1;
  }
  return v;
}

int launch_batch(bool apply, int count, const void* d_desc, int n_ids, int n_tasks, size_t smem,
                 int ctas_per_sm, DagWorkspace* ws, long long timeout_ns, cudaStream_t stream) {
  if (count <= 0 || n_tasks <= 0) return HQR_ERR_INVALID;
  DagParams p{};
  p.mode = apply ? kModeApplyQt : kModeFactor;
  p.skip_panels = apply ? 1 : 0;
  p.n_mats = count;
  p.mats = static_cast<const MatDesc*>(d_desc);
  p.n_ids = n_ids;
  p.n_tasks = n_tasks;
  p.timeout_ns = timeout_ns;
  int rc = dag_workspace_reserve(ws, (size_t)n_ids);
  if (rc != HQR_OK) return rc;
  p.cnt = ws->cnt;
  p.qhi = ws->qhi;
  p.qlo = ws->qlo;
  p.ctl = ws->ctl;
  p.stats = ws->stats;
  cudaError_t e = cudaMemsetAsync(ws->ctl, 0, kErr * sizeof(unsigned), stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(ws->stats, 0, 2 * kNumStats * sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return record_cuda_error(e, "DAG workspace reset");
  static SmemOptIn opted;
  int occ = 1;
  e = opt_in(opted, dag_exec_kernel<false, true>, smem, [] {
    return cudaFuncSetAttribute(dag_exec_kernel<false, true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                (int)cudaSharedmemCarveoutMaxShared);
  });
  if (e != cudaSuccess) return record_cuda_error(e, "cudaFuncSetAttribute(dag_exec_kernel batch)");
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, dag_exec_kernel<false, true>, kThreads, smem);
  if (e != cudaSuccess) return record_cuda_error(e, "occupancy of dag_exec_kernel batch");
  if (occ < 1) return HQR_ERR_UNSUPPORTED;
  if (ctas_per_sm > 0) occ = std::min(occ, ctas_per_sm);
  dag_init_batch_kernel<<<count, 256, 0, stream>>>(p);
  dag_seed_batch_kernel<<<count, 256, 0, stream>>>(p);
  const int grid = std::min(occ * dag_sm_count(), std::max(1, n_tasks));
  dag_exec_kernel<false, true><<<grid, kThreads, smem, stream>>>(p);
  e = cudaGetLastError();
  if (e != cudaSuccess) return record_cuda_error(e, "dag_exec_kernel batch launch");
  return HQR_OK;
}

bool oz_supported(const Geometry& g) { return g.NB == oz::kK; }

// The split path rebuilds every panel tile's full T from V and TAU, which do
// not depend on the inner block width of the FP64 panels: those run with the
// narrower w = 16, whose column loop is shorter (about 13 % faster GEQRT and
// TSQRT at NB = 128, the factorization's critical path).
int narrow_panels(Geometry* g) {
  if (g->w <= 16) return HQR_OK;
  g->w = 16;
  const SmemPlan sp = SmemPlan::make(shape_of(*g));
  g->smem_bytes = (size_t)sp.total * sizeof(double);
  return HQR_OK;
}

static size_t panel_tiles(const Geometry& g) {
  return panel_slot(g.MT, g.steps, g.steps);   // slots of every (k, i), k >= i, i < steps
}
size_t oz_slice_bytes(const Geometry& g) { return panel_tiles(g) * oz::panel_slice_bytes(); }
size_t oz_panel_bytes() { return oz::panel_slice_bytes(); }
size_t oz_exp_bytes(const Geometry& g) { return panel_tiles(g) * oz::kSlots * (size_t)g.NB * sizeof(int); }
size_t oz_exp_bytes_per_panel(int NB) { return (size_t)oz::kSlots * NB * sizeof(int); }

size_t tree_slots(const Geometry& g, int S) {
  if (S <= 0 || S >= g.MT) return 0;
  return (size_t)g.steps * ((g.MT + S - 1) / S);
}

size_t factor_task_ids(const Geometry& g) {
  return (size_t)g.steps * g.MT * (g.NB / g.w) + (size_t)g.steps * g.NT * g.MT * g.NC;
}

int launch_factor_external(const Geometry& g, const ExternalScratch& x, double* dA, double* dTAU,
                           long long timeout_ns, cudaStream_t stream) {
  static_assert(kExternalCtlBytes == kCtlWords * sizeof(unsigned), "control words");
  static_assert(kExternalStatsBytes == 2 * kNumStats * sizeof(unsigned long long), "stats");
  DagParams p{};
  p.mode = kModeFactor;
  p.MT = g.MT;
  p.NT = g.NT;
  p.CT = g.NT;
  p.NC = g.NC;
  p.steps = g.steps;
  p.J = g.NT;
  p.nblk = g.NB / g.w;
  p.sh = shape_of(g);
  p.sp = SmemPlan::make(p.sh);
  p.n_ids = (int)factor_task_ids(g);
  long long n = 0;
  for (int i = 0; i < g.steps; i++)
    n += (long long)(g.MT - i) * p.nblk + (long long)g.NC * (g.NT - 1 - i) * (g.MT - i);
  p.n_tasks = (int)n;
  p.A = dA;
  p.T = x.T;
  p.TAU = dTAU;
  p.C = dA;
  p.cnt = x.cnt;
  p.qhi = x.qhi;
  p.qlo = x.qlo;
  p.ctl = x.ctl;
  p.stats = x.stats;
  p.timeout_ns = timeout_ns;
  static SmemOptIn opted;
  {
    const cudaError_t e = opt_in(opted, dag_exec_kernel<false>, g.smem_bytes);
    if (e != cudaSuccess) return record_cuda_error(e, "cudaFuncSetAttribute(dag_exec_kernel)");
  }
  const int blocks = (p.n_ids + 255) / 256;
  dag_init_kernel<<<blocks, 256, 0, stream>>>(p);
  dag_seed_kernel<<<blocks, 256, 0, stream>>>(p);
  const int grid = std::min(dag_sm_count(), std::max(1, p.n_tasks));
  dag_exec_kernel<false><<<grid, kThreads, g.smem_bytes, stream>>>(p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return record_cuda_error(e, "dag_exec_kernel launch");
  return HQR_OK;
}

int external_status(const ExternalScratch& x, cudaStream_t stream) {
  unsigned ctl[kCtlWords];
  cudaError_t e = cudaMemcpyAsync(ctl, x.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return record_cuda_error(e, "DAG execution (stream synchronize)");
  if (ctl[kErr] != 0u) return (ctl[kErr] & kErrTimeout) ? HQR_ERR_TIMEOUT : HQR_ERR_DEVICE;
  return HQR_OK;
}

int dag_status(DagWorkspace* ws, cudaStream_t stream) {
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return record_cuda_error(e, "DAG execution (stream synchronize)");
  unsigned ctl[kCtlWords];
  e = cudaMemcpy(ctl, ws->ctl, sizeof(ctl), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return record_cuda_error(e, "DAG status read");
  if (ctl[kErr] != 0u) {
    cudaMemset(ws->ctl + kErr, 0, sizeof(unsigned));
    if (ctl[kErr] & kErrTimeout) return HQR_ERR_TIMEOUT;
    return HQR_ERR_DEVICE;
  }
  return HQR_OK;
}

int dag_stats(DagWorkspace* ws, unsigned long long out[14], cudaStream_t stream) {
  if (cudaStreamSynchronize(stream) != cudaSuccess) return HQR_ERR_CUDA;
  if (cudaMemcpy(out, ws->stats, 14 * sizeof(unsigned long long), cudaMemcpyDeviceToHost) !=
      cudaSuccess)
    return HQR_ERR_CUDA;
  return HQR_OK;
}

}  // namespace hqr
