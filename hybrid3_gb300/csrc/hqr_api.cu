// hqr_api.cu -- the library's C ABI: the extended device API of hqr_gpu.h and
// the drop-in Hybrid_* entry points of Hybrid_tile_QR.h.
//
// The drop-in functions keep the reference's calling convention (host arrays
// in tile layout, void return, abort on error -- Hybrid_tile_QR.c:992-999 and
// friends call MPI_Abort): each call stages its operands in device buffers
// owned by the library, runs the tile DAG on the GPU and copies results back.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "Hybrid_tile_QR.h"
#include "hqr_internal.h"

struct hqr_plan {
  hqr::Geometry g;
  int precision;
  double* dT;
  hqr::DagWorkspace ws;
  hqr::OzWorkspace oz;   // allocated for the split precisions only
  hqr::TreeWorkspace tree;   // domain tree (hqr_plan_set_tree); S = 0: flat
  // split precisions: the prepared operands of H itself (Q generation, Q C),
  // allocated on first use; oz holds those of H^T (factorization, Q^T C)
  hqr::OzWorkspace ozh;
  // 1 while dT / oz (h_valid: ozh) hold the T factors / prepared operands of
  // the last factorization on this plan (a rebuild from other reflectors
  // replaces them)
  int factors_valid = 0;
  int h_valid = 0;
  // least-squares workspace (hqr_lstsq, hqr_lstsq_aug), grow-only, kept
  // between calls so that a solve allocates nothing after the first
  double* ls[9] = {};
  size_t ls_cap[9] = {};
};

namespace {

int g_error_mode = HQR_ERRORS_ABORT;
int g_default_precision = -1;   // -1: not chosen yet (HQR_PRECISION, else FP64)
thread_local int g_last_error = HQR_OK;
long long g_timeout_ns = 20000LL * 1000000LL;
std::mutex g_mu;   // serialises the drop-in entry points (they share buffers)
char g_cuda_msg[256] = "";

int cuda_rc(cudaError_t e) {
  return e == cudaSuccess ? HQR_OK : hqr::record_cuda_error(e, "CUDA runtime call");
}

// Device buffers reused across drop-in calls (grow-only).
struct Staging {
  double* buf[4] = {nullptr, nullptr, nullptr, nullptr};
  size_t cap[4] = {0, 0, 0, 0};
  cudaStream_t stream = nullptr;
  cudaEvent_t h2d_done = nullptr;   // recorded after a call's host-to-device copies
  hqr_plan* plan = nullptr;
};
Staging g_stage;

int stage_reserve(int slot, size_t n_doubles, double** out) {
  if (g_stage.cap[slot] < n_doubles) {
    if (g_stage.buf[slot]) cudaFree(g_stage.buf[slot]);
    g_stage.buf[slot] = nullptr;
    g_stage.cap[slot] = 0;
    if (cudaMalloc(&g_stage.buf[slot], n_doubles * sizeof(double)) != cudaSuccess)
      return HQR_ERR_NOMEM;
    g_stage.cap[slot] = n_doubles;
  }
  *out = g_stage.buf[slot];
  return HQR_OK;
}

int stage_stream(cudaStream_t* s) {
  if (!g_stage.stream) {
    if (cudaStreamCreateWithFlags(&g_stage.stream, cudaStreamNonBlocking) != cudaSuccess)
      return HQR_ERR_CUDA;
  }
  if (!g_stage.h2d_done && cudaEventCreateWithFlags(&g_stage.h2d_done, cudaEventDisableTiming) != cudaSuccess)
    return HQR_ERR_CUDA;
  *s = g_stage.stream;
  return HQR_OK;
}

// Hybrid_remv_Y on a host array in tile layout (what the device's
// zero_reflectors does): the strictly lower triangle of each diagonal tile and
// every tile below it, in the first min(MT, NT) tile columns.  Host threads
// take tile columns from a shared counter.
void host_zero_reflectors(double* A, long M, long N, int NB) {
  const int MT = (int)(M / NB), NT = (int)(N / NB), steps = std::min(MT, NT);
  const size_t tsz = (size_t)NB * NB;
  std::atomic<int> next{0};
  auto work = [&]() {
    for (int tj; (tj = next.fetch_add(1)) < steps;) {
      double* col = A + (size_t)tj * MT * tsz;   // tile (0, tj)
      double* d = col + (size_t)tj * tsz;
      for (int c = 0; c + 1 < NB; c++) memset(d + (size_t)c * NB + c + 1, 0, (size_t)(NB - c - 1) * sizeof(double));
      if (tj + 1 < MT) memset(col + (size_t)(tj + 1) * tsz, 0, (size_t)(MT - tj - 1) * tsz * sizeof(double));
    }
  };
  const unsigned hw = std::thread::hardware_concurrency();
  const int nt = (int)std::min<unsigned>(16u, std::max(1u, std::min<unsigned>(hw, (unsigned)steps)));
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; t++) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
}

// Plan for the drop-in calls, rebuilt when the shape changes.
int stage_plan(long M, long N, int NB, int IB, hqr_plan** out) {
  hqr_plan* p = g_stage.plan;
  if (p && p->g.M == M && p->g.N == N && p->g.NB == NB && p->g.IB == IB &&
      p->precision == hqr_get_default_precision()) {
    *out = p;
    return HQR_OK;
  }
  if (p) hqr_plan_destroy(p);
  g_stage.plan = nullptr;
  int rc = hqr_plan_create(&g_stage.plan, M, N, NB, IB, hqr_get_default_precision());
  *out = g_stage.plan;
  return rc;
}

int report(const char* fn, int rc) {
  g_last_error = rc;
  if (rc == HQR_OK) return rc;
  fprintf(stderr, "hybrid3_gb300: %s: %s%s%s\n", fn, hqr_status_string(rc),
          rc == HQR_ERR_CUDA ? " -- " : "", rc == HQR_ERR_CUDA ? g_cuda_msg : "");
  if (g_error_mode == HQR_ERRORS_ABORT) {
    fflush(stderr);
    exit(1);
  }
  return rc;
}

int check_status(const mat_stat_t* st, int my_rank, int Proc_num) {
  if (!st) return HQR_ERR_INVALID;
  if (Proc_num != 1 || my_rank != 0) return HQR_ERR_INVALID;
  if (st->tile_M != st->tile_N || st->tile_M == 0) return HQR_ERR_INVALID;
  if (st->my_mat_M != (unsigned long)st->my_tile_M * st->tile_M) return HQR_ERR_INVALID;
  if (st->my_mat_N != (unsigned long)st->my_tile_N * st->tile_N) return HQR_ERR_INVALID;
  return HQR_OK;
}

size_t tau_len(const hqr::Geometry& g) { return (size_t)g.MT * g.NT * g.NB; }

bool split_precision(int precision) {
  return precision == HQR_PREC_OZAKI || precision == HQR_PREC_OZAKI_FAST || precision == HQR_PREC_FP32;
}

#define TRY(x)                      \
  do {                              \
    int _rc = (x);                  \
    if (_rc != HQR_OK) return _rc;  \
  } while (0)

// Q^T into dQ, which the caller has zeroed (Hybrid_make_Q.c:91-95 sets the
// diagonal of a caller-zeroed Q and applies H_1^T ... H_k^T to it).  Square
// matrices: Q = H_1 (H_2 (... (H_k I))) accumulated backwards, which skips the
// tile columns that are still unit vectors (2/3 of the forward updates), then
// transposed in place; the identity is written whole, so the result does not
// depend on dQ's prior contents.  Other shapes: the forward application.
// The T factors (FP64: one set for both directions) or prepared operands
// (split: the H^T set oz, or with h the H set ozh) a Q application uses, and
// whether its panel tasks rebuild them from the given reflectors.  plan_refl:
// the caller vouches that those are the last factorization's on this plan
// (use_plan_t); they are then rebuilt only if a rebuild from other reflectors
// has replaced them, and are valid again afterwards.  Null: no memory for ozh.
const hqr::OzWorkspace* apply_operands(hqr_plan* plan, bool h, bool plan_refl, bool* rebuild) {
  const bool split = plan->oz.slices != nullptr;
  if (split && h && !plan->ozh.slices) {
    plan->ozh.groups = plan->oz.groups;
    plan->ozh.fp32_panels = plan->oz.fp32_panels;
    if (cudaMalloc(&plan->ozh.slices, hqr::oz_slice_bytes(plan->g)) != cudaSuccess ||
        cudaMalloc(&plan->ozh.sexp, hqr::oz_exp_bytes(plan->g)) != cudaSuccess) {
      cudaFree(plan->ozh.slices);
      plan->ozh = hqr::OzWorkspace{};
      return nullptr;
    }
  }
  int* valid = (split && h) ? &plan->h_valid : &plan->factors_valid;
  *rebuild = !plan_refl || !*valid;
  if (*rebuild) *valid = plan_refl ? 1 : 0;
  return (split && h) ? &plan->ozh : &plan->oz;
}

// dQ <- Q^T of the factorization (dRY, dTAU); plan_refl as for apply_operands.
// untransposed (square matrices): if not null, the backward accumulation
// leaves Q itself in dQ and *untransposed is set; the caller transposes it.
int build_qt(hqr_plan* plan, double* dQ, const double* dRY, const double* dTAU, bool plan_refl,
             cudaStream_t s) {
  const hqr::Geometry& g = plan->g;
  if (plan->tree.S > 0) {   // a tree's merges live in the plan: forward application on I
    if (!plan_refl) return HQR_ERR_UNSUPPORTED;
    hqr::make_identity(dQ, g.M, g.N, g.NB, true, s);
    return hqr::launch_apply_qt_tree(g, &plan->ws, dRY, plan->dT, dTAU, dQ, g.NT, g_timeout_ns, s,
                                     &plan->oz, &plan->tree);
  }
  bool rebuild;
  if (g.M == g.N && g.NB % 32 == 0) {
    // backward accumulation Q = H_0 (H_1 (... I)): H itself
    const hqr::OzWorkspace* oz = apply_operands(plan, true, plan_refl, &rebuild);
    if (!oz) return HQR_ERR_NOMEM;
    hqr::make_identity(dQ, g.M, g.N, g.NB, true, s);
    TRY(hqr::launch_build_q(g, &plan->ws, dRY, plan->dT, dTAU, dQ, rebuild, g_timeout_ns, s, oz));
    hqr::transpose_tiles(dQ, g.N, g.NB, s);
    return cuda_rc(cudaGetLastError());
  }
  const hqr::OzWorkspace* oz = apply_operands(plan, false, plan_refl, &rebuild);
  hqr::make_identity(dQ, g.M, g.N, g.NB, false, s);
  return hqr::launch_apply_qt(g, &plan->ws, dRY, plan->dT, dTAU, dQ, g.NT, rebuild, g_timeout_ns, s, oz);
}

// Phases of the last drop-in call, from CUDA events on the staging stream:
// marks 0..4 = before the host-to-device copies, after them, after the DAG
// launch(es) were enqueued, after the host read the scheduler's status, after
// the device-to-host copies.
struct PhaseTimes {
  cudaEvent_t ev[5] = {};
  bool ready = false;
  double ms[6] = {};
  std::chrono::steady_clock::time_point t0;
};
PhaseTimes g_phase;

void phase_begin(cudaStream_t s) {
  if (!g_phase.ready) {
    g_phase.ready = true;
    for (auto& e : g_phase.ev)
      if (cudaEventCreate(&e) != cudaSuccess) g_phase.ready = false;
  }
  g_phase.t0 = std::chrono::steady_clock::now();
  if (g_phase.ready) cudaEventRecord(g_phase.ev[0], s);
}
void phase_mark(int i, cudaStream_t s) {
  if (g_phase.ready) cudaEventRecord(g_phase.ev[i], s);
}
// After the final synchronisation: [h2d, DAG, idle while the host checked the
// status, d2h, device total, host wall time] in milliseconds.
void phase_end() {
  const double host = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - g_phase.t0).count();
  if (!g_phase.ready) return;
  float f[5] = {0, 0, 0, 0, 0};
  for (int i = 0; i < 4; i++) cudaEventElapsedTime(&f[i], g_phase.ev[i], g_phase.ev[i + 1]);
  cudaEventElapsedTime(&f[4], g_phase.ev[0], g_phase.ev[4]);
  for (int i = 0; i < 5; i++) g_phase.ms[i] = f[i];
  g_phase.ms[5] = host;
}

int h2d(double* d, const double* h, size_t n, cudaStream_t s) {
  return cuda_rc(hqr::copy_host_to_device(d, h, n, s));
}
int d2h(double* h, const double* d, size_t n, cudaStream_t s) {
  return cuda_rc(hqr::copy_device_to_host(h, d, n, s));
}

}  // namespace

int hqr::report_error(const char* fn, int rc) { return report(fn, rc); }

int hqr::record_cuda_error(cudaError_t e, const char* where) {
  snprintf(g_cuda_msg, sizeof(g_cuda_msg), "%s: %s (%d)", where, cudaGetErrorString(e), (int)e);
  return HQR_ERR_CUDA;
}

// ===========================================================================
// Extended API
// ===========================================================================
extern "C" {

const char* hqr_status_string(int s) {
  switch (s) {
    case HQR_OK: return "ok";
    case HQR_ERR_INVALID: return "invalid argument";
    case HQR_ERR_CUDA: return "CUDA runtime error";
    case HQR_ERR_TIMEOUT: return "device scheduler wait timed out";
    case HQR_ERR_NOMEM: return "device allocation failed";
    case HQR_ERR_UNSUPPORTED: return "unsupported shape";
    case HQR_ERR_DEVICE: return "device-side consistency check failed";
    default: return "unknown status";
  }
}

void hqr_set_error_mode(int mode) { g_error_mode = mode; }

int hqr_get_default_precision(void) {
  if (g_default_precision < 0) {
    const char* e = getenv("HQR_PRECISION");
    g_default_precision = (e && (!strcmp(e, "ozaki") || !strcmp(e, "split")))  ? HQR_PREC_OZAKI
                          : (e && !strcmp(e, "fast"))                             ? HQR_PREC_OZAKI_FAST
                          : (e && !strcmp(e, "fp32"))                             ? HQR_PREC_FP32
                                                                                  : HQR_PREC_FP64;
  }
  return g_default_precision;
}
void hqr_set_default_precision(int precision) {
  g_default_precision = split_precision(precision) ? precision : HQR_PREC_FP64;
}
int hqr_last_error(void) { return g_last_error; }
const char* hqr_last_cuda_error(void) { return g_cuda_msg; }
void hqr_set_timeout_ms(long long ms) { g_timeout_ns = (ms > 0 ? ms : 1) * 1000000LL; }

int hqr_plan_create(hqr_plan_t** plan, long M, long N, int NB, int IB, int precision) {
  if (!plan) return HQR_ERR_INVALID;
  *plan = nullptr;
  if (precision != HQR_PREC_FP64 && !split_precision(precision)) return HQR_ERR_INVALID;
  hqr::Geometry g;
  TRY(hqr::make_geometry(M, N, NB, IB, &g));
  if (split_precision(precision) && !hqr::oz_supported(g)) return HQR_ERR_UNSUPPORTED;
  if (split_precision(precision)) TRY(hqr::narrow_panels(&g));
  hqr_plan* p = new hqr_plan();
  p->g = g;
  p->precision = precision;
  p->dT = nullptr;
  if (cudaMalloc(&p->dT, (size_t)M * N * sizeof(double)) != cudaSuccess) {
    delete p;
    return HQR_ERR_NOMEM;
  }
  cudaMemset(p->dT, 0, (size_t)M * N * sizeof(double));
  if (split_precision(precision)) {
    p->oz.groups = precision == HQR_PREC_OZAKI ? 8 : 4;
    p->oz.fp32_panels = precision == HQR_PREC_FP32 ? 1 : 0;
    if (cudaMalloc(&p->oz.slices, hqr::oz_slice_bytes(g)) != cudaSuccess ||
        cudaMalloc(&p->oz.sexp, hqr::oz_exp_bytes(g)) != cudaSuccess) {
      hqr_plan_destroy(p);
      return HQR_ERR_NOMEM;
    }
  }
  *plan = p;
  return HQR_OK;
}

namespace {
void free_tree(hqr::TreeWorkspace* t) {
  cudaFree(t->T2);
  cudaFree(t->TAU2);
  cudaFree(t->slices2);
  cudaFree(t->sexp2);
  *t = hqr::TreeWorkspace{};
}
}  // namespace

int hqr_plan_set_tree(hqr_plan_t* plan, int domain_tiles) {
  if (!plan || domain_tiles < 0) return HQR_ERR_INVALID;
  free_tree(&plan->tree);
  const hqr::Geometry& g = plan->g;
  const size_t slots = hqr::tree_slots(g, domain_tiles);
  if (slots == 0) return HQR_OK;   // one domain: the flat tree
  // the task ids of the tree DAG must fit an int
  const long long dmax = (g.MT + domain_tiles - 1) / domain_tiles;
  const long long extra = (long long)g.steps * dmax * ((long long)g.NB / g.w + 1 + (long long)g.NT * 2);
  if (extra > 0x1fffffffLL) return HQR_ERR_UNSUPPORTED;
  hqr::TreeWorkspace t;
  t.S = domain_tiles;
  const size_t nb = (size_t)g.NB;
  bool ok = cudaMalloc(&t.T2, slots * nb * nb * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&t.TAU2, slots * nb * sizeof(double)) == cudaSuccess;
  if (ok && split_precision(plan->precision))
    ok = cudaMalloc(&t.slices2, slots * hqr::oz_panel_bytes()) == cudaSuccess &&
         cudaMalloc(&t.sexp2, slots * hqr::oz_exp_bytes_per_panel((int)nb)) == cudaSuccess;
  if (!ok) {
    free_tree(&t);
    return HQR_ERR_NOMEM;
  }
  cudaMemset(t.T2, 0, slots * nb * nb * sizeof(double));
  plan->tree = t;
  return HQR_OK;
}

int hqr_plan_destroy(hqr_plan_t* plan) {
  if (!plan) return HQR_ERR_INVALID;
  free_tree(&plan->tree);
  if (plan->dT) cudaFree(plan->dT);
  if (plan->oz.slices) cudaFree(plan->oz.slices);
  if (plan->oz.sexp) cudaFree(plan->oz.sexp);
  if (plan->ozh.slices) cudaFree(plan->ozh.slices);
  if (plan->ozh.sexp) cudaFree(plan->ozh.sexp);
  hqr::dag_workspace_free(&plan->ws);
  for (double* p : plan->ls) cudaFree(p);
  delete plan;
  return HQR_OK;
}

double* hqr_plan_t_factors(hqr_plan_t* plan) { return plan ? plan->dT : nullptr; }

int hqr_geqrf_async(hqr_plan_t* plan, double* dA, double* dTAU, void* stream) {
  if (!plan || !dA || !dTAU) return HQR_ERR_INVALID;
  plan->factors_valid = 0;
  plan->h_valid = 0;
  TRY(hqr::launch_factor(plan->g, &plan->ws, dA, plan->dT, dTAU, g_timeout_ns, (cudaStream_t)stream, &plan->oz,
                         &plan->tree));
  plan->factors_valid = 1;
  return HQR_OK;
}

int hqr_plan_status(hqr_plan_t* plan, void* stream) {
  if (!plan) return HQR_ERR_INVALID;
  if (!plan->ws.ctl) return cuda_rc(cudaStreamSynchronize((cudaStream_t)stream));
  return hqr::dag_status(&plan->ws, (cudaStream_t)stream);
}

int hqr_geqrf(hqr_plan_t* plan, double* dA, double* dTAU, void* stream) {
  TRY(hqr_geqrf_async(plan, dA, dTAU, stream));
  return hqr_plan_status(plan, stream);
}

int hqr_plan_stats(hqr_plan_t* plan, hqr_stats_t* out, void* stream) {
  if (!plan || !out || !plan->ws.stats) return HQR_ERR_INVALID;
  unsigned long long v[14];
  TRY(hqr::dag_stats(&plan->ws, v, (cudaStream_t)stream));
  for (int t = 0; t < 7; t++) {
    out->count[t] = v[2 * t];
    out->cycles[t] = v[2 * t + 1];
  }
  return HQR_OK;
}

int hqr_make_q_async(hqr_plan_t* plan, double* dQ, double* dRY, const double* dTAU, int use_plan_t,
                     void* stream) {
  if (!plan || !dQ || !dRY || !dTAU) return HQR_ERR_INVALID;
  const hqr::Geometry& g = plan->g;
  cudaStream_t s = (cudaStream_t)stream;
  TRY(build_qt(plan, dQ, dRY, dTAU, use_plan_t != 0, s));
  hqr::zero_reflectors(dRY, g.M, g.N, g.NB, s);
  return cuda_rc(cudaGetLastError());
}

int hqr_make_q(hqr_plan_t* plan, double* dQ, double* dRY, const double* dTAU, int use_plan_t,
               void* stream) {
  TRY(hqr_make_q_async(plan, dQ, dRY, dTAU, use_plan_t, stream));
  return hqr_plan_status(plan, stream);
}

namespace {
// Q^T C and Q C on C's first ccols columns (0: all CT tile columns); the
// columns beyond are zero and stay so.
int ormqr_t_cols(hqr_plan_t* plan, const double* dRY, const double* dTAU, double* dC, int CT, int use_plan_t,
                 cudaStream_t s, long long ccols) {
  if (!plan || !dRY || !dTAU || !dC || CT <= 0) return HQR_ERR_INVALID;
  if (plan->tree.S > 0) {
    if (!use_plan_t) return HQR_ERR_UNSUPPORTED;   // the merges' T factors live in the plan
    return hqr::launch_apply_qt_tree(plan->g, &plan->ws, dRY, plan->dT, dTAU, dC, CT, g_timeout_ns, s,
                                     &plan->oz, &plan->tree);
  }
  bool rebuild;
  const hqr::OzWorkspace* oz = apply_operands(plan, false, use_plan_t != 0, &rebuild);
  return hqr::launch_apply_qt(plan->g, &plan->ws, dRY, plan->dT, dTAU, dC, CT, rebuild, g_timeout_ns, s, oz,
                              ccols);
}
int ormqr_n_cols(hqr_plan_t* plan, const double* dRY, const double* dTAU, double* dC, int CT, int use_plan_t,
                 cudaStream_t s, long long ccols) {
  if (!plan || !dRY || !dTAU || !dC || CT <= 0) return HQR_ERR_INVALID;
  if (plan->tree.S > 0) return HQR_ERR_UNSUPPORTED;
  bool rebuild;
  const hqr::OzWorkspace* oz = apply_operands(plan, true, use_plan_t != 0, &rebuild);
  if (!oz) return HQR_ERR_NOMEM;
  return hqr::launch_apply_q(plan->g, &plan->ws, dRY, plan->dT, dTAU, dC, CT, rebuild, g_timeout_ns, s, oz,
                             ccols);
}
}  // namespace

int hqr_ormqr_t_async(hqr_plan_t* plan, const double* dRY, const double* dTAU, double* dC, int CT,
                      int use_plan_t, void* stream) {
  return ormqr_t_cols(plan, dRY, dTAU, dC, CT, use_plan_t, (cudaStream_t)stream, 0);
}

int hqr_ormqr_t(hqr_plan_t* plan, const double* dRY, const double* dTAU, double* dC, int CT,
                int use_plan_t, void* stream) {
  TRY(hqr_ormqr_t_async(plan, dRY, dTAU, dC, CT, use_plan_t, stream));
  return hqr_plan_status(plan, stream);
}

int hqr_ormqr_n_async(hqr_plan_t* plan, const double* dRY, const double* dTAU, double* dC, int CT,
                      int use_plan_t, void* stream) {
  return ormqr_n_cols(plan, dRY, dTAU, dC, CT, use_plan_t, (cudaStream_t)stream, 0);
}

int hqr_ormqr_n(hqr_plan_t* plan, const double* dRY, const double* dTAU, double* dC, int CT, int use_plan_t,
                void* stream) {
  TRY(hqr_ormqr_n_async(plan, dRY, dTAU, dC, CT, use_plan_t, stream));
  return hqr_plan_status(plan, stream);
}

namespace {
// The plan's least-squares buffers.
enum LsBuf {
  kLsAf,    // the factored copy of A
  kLsTau,
  kLsC,     // right-hand sides / residuals in tile layout
  kLsG,     // [h; d2] in tile layout, then the residual's correction (augmented)
  kLsRes,   // b - A x, column-major M x nrhs
  kLsR,     // the refined least-squares residual r, column-major M x nrhs (augmented)
  kLsAtr,   // -A^T r, column-major N x nrhs (augmented)
  kLsPart,  // partial sums of A^T r (augmented)
  kLsNrm,
};
int ls_buf(hqr_plan* plan, LsBuf which, size_t n, double** out) {
  if (plan->ls_cap[which] < n) {
    cudaFree(plan->ls[which]);
    plan->ls[which] = nullptr;
    plan->ls_cap[which] = 0;
    if (cudaMalloc(&plan->ls[which], n * sizeof(double)) != cudaSuccess) return HQR_ERR_NOMEM;
    plan->ls_cap[which] = n;
  }
  *out = plan->ls[which];
  return HQR_OK;
}

// Common start of both solves: A copied and factored, x0 = R^-1 (Q^T b)(1:N)
// in dX; all enqueued on s.
int ls_start(hqr_plan* plan, const double* dA, const double* dB, int ldb, int nrhs, double* dX, int ldx,
             double* Af, double* tau, double* C, cudaStream_t s) {
  const hqr::Geometry& g = plan->g;
  const int CT = (nrhs + g.NB - 1) / g.NB;
  TRY(cuda_rc(cudaMemcpyAsync(Af, dA, (size_t)g.M * g.N * sizeof(double), cudaMemcpyDeviceToDevice, s)));
  TRY(hqr_geqrf_async(plan, Af, tau, s));
  hqr::pack_rhs(dB, ldb, nrhs, C, g.M, g.NB, CT, s);
  TRY(cuda_rc(cudaGetLastError()));
  TRY(ormqr_t_cols(plan, Af, tau, C, CT, 1, s, nrhs));
  TRY(hqr::trsm_tiles(Af, g.M, g.N, g.NB, C, nrhs, s));
  hqr::update_x(C, g.M, g.NB, g.N, nrhs, dX, ldx, false, s);
  return cuda_rc(cudaGetLastError());
}

// End of both solves: the scheduler's status, then ||b - A x||_2 per
// right-hand side into resid (host) if it is not null.
int ls_finish(hqr_plan* plan, const double* dA, const double* dB, int ldb, int nrhs, const double* dX,
              int ldx, double* Res, double* nrm, double* resid, cudaStream_t s) {
  const hqr::Geometry& g = plan->g;
  if (resid) {
    TRY(hqr::residual(dA, g.M, g.N, g.NB, dX, ldx, dB, ldb, Res, g.M, nrhs, s));
    hqr::col_norm2(Res, g.M, g.M, nrhs, nrm, s);
    TRY(cuda_rc(cudaMemcpyAsync(resid, nrm, (size_t)nrhs * sizeof(double), cudaMemcpyDeviceToHost, s)));
  }
  TRY(hqr_plan_status(plan, s));
  if (resid)
    for (int q = 0; q < nrhs; q++) resid[q] = sqrt(resid[q]);
  return HQR_OK;
}
}  // namespace

int hqr_lstsq(hqr_plan_t* plan, const double* dA, const double* dB, int ldb, int nrhs, double* dX,
              int ldx, int refine_steps, double* resid, void* stream) {
  if (!plan || !dA || !dB || !dX || nrhs <= 0 || refine_steps < 0) return HQR_ERR_INVALID;
  const hqr::Geometry& g = plan->g;
  if (g.M < g.N || ldb < g.M || ldx < g.N) return HQR_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const int CT = (nrhs + g.NB - 1) / g.NB;
  double *Af, *tau, *C, *Res, *nrm;
  TRY(ls_buf(plan, kLsAf, (size_t)g.M * g.N, &Af));
  TRY(ls_buf(plan, kLsTau, tau_len(g), &tau));
  TRY(ls_buf(plan, kLsC, (size_t)g.M * CT * g.NB, &C));
  TRY(ls_buf(plan, kLsRes, (size_t)g.M * nrhs, &Res));
  TRY(ls_buf(plan, kLsNrm, (size_t)nrhs, &nrm));
  TRY(ls_start(plan, dA, dB, ldb, nrhs, dX, ldx, Af, tau, C, s));
  for (int it = 1; it <= refine_steps; it++) {
    TRY(hqr::residual(dA, g.M, g.N, g.NB, dX, ldx, dB, ldb, Res, g.M, nrhs, s));
    hqr::pack_rhs(Res, g.M, nrhs, C, g.M, g.NB, CT, s);
    TRY(cuda_rc(cudaGetLastError()));
    TRY(ormqr_t_cols(plan, Af, tau, C, CT, 1, s, nrhs));
    TRY(hqr::trsm_tiles(Af, g.M, g.N, g.NB, C, nrhs, s));
    hqr::update_x(C, g.M, g.NB, g.N, nrhs, dX, ldx, true, s);
    TRY(cuda_rc(cudaGetLastError()));
  }
  return ls_finish(plan, dA, dB, ldb, nrhs, dX, ldx, Res, nrm, resid, s);
}

// Bjorck's refinement on the augmented system [I A; A^T 0][r; x] = [b; 0]:
// each step forms f = b - r - A x and g = -A^T r in FP64 and solves the
// correction system with the factorization -- h = R^-T g, d = Q^T f,
// dx = R^-1 (d(1:N) - h), dr = Q [h; d(N+1:M)] -- so the floor of x is set by
// the FP64 residuals (kappa u), not by the factorization's precision.
int hqr_lstsq_aug(hqr_plan_t* plan, const double* dA, const double* dB, int ldb, int nrhs, double* dX,
                  int ldx, int refine_steps, double* resid, void* stream) {
  if (!plan || !dA || !dB || !dX || nrhs <= 0 || refine_steps < 0) return HQR_ERR_INVALID;
  const hqr::Geometry& g = plan->g;
  if (g.M < g.N || ldb < g.M || ldx < g.N) return HQR_ERR_INVALID;
  if (plan->tree.S > 0) return HQR_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  const int CT = (nrhs + g.NB - 1) / g.NB;
  const int S = hqr::atr_slices(g.M, g.N, g.NB, nrhs);
  double *Af, *tau, *C, *G, *Res, *r, *atr, *part, *nrm;
  TRY(ls_buf(plan, kLsAf, (size_t)g.M * g.N, &Af));
  TRY(ls_buf(plan, kLsTau, tau_len(g), &tau));
  TRY(ls_buf(plan, kLsC, (size_t)g.M * CT * g.NB, &C));
  TRY(ls_buf(plan, kLsG, (size_t)g.M * CT * g.NB, &G));
  TRY(ls_buf(plan, kLsRes, (size_t)g.M * nrhs, &Res));
  TRY(ls_buf(plan, kLsR, (size_t)g.M * nrhs, &r));
  TRY(ls_buf(plan, kLsAtr, (size_t)g.N * nrhs, &atr));
  TRY(ls_buf(plan, kLsPart, (size_t)S * g.N * nrhs, &part));
  TRY(ls_buf(plan, kLsNrm, (size_t)nrhs, &nrm));
  TRY(ls_start(plan, dA, dB, ldb, nrhs, dX, ldx, Af, tau, C, s));
  TRY(hqr::residual(dA, g.M, g.N, g.NB, dX, ldx, dB, ldb, r, g.M, nrhs, s));   // r0 = b - A x0
  const int MT = (int)(g.M / g.NB), NT = (int)(g.N / g.NB);
  for (int it = 0; it < refine_steps; it++) {
    // f = b - A x - r, g = -A^T r
    TRY(hqr::residual(dA, g.M, g.N, g.NB, dX, ldx, dB, ldb, Res, g.M, nrhs, s));
    hqr::sub_colmajor(Res, g.M, r, g.M, g.M, nrhs, s);
    TRY(hqr::at_times(dA, g.M, g.N, g.NB, r, g.M, nrhs, -1.0, atr, g.N, part, S, s));
    // d = Q^T f; h = R^-T g
    hqr::pack_rhs(Res, g.M, nrhs, C, g.M, g.NB, CT, s);
    TRY(cuda_rc(cudaGetLastError()));
    TRY(ormqr_t_cols(plan, Af, tau, C, CT, 1, s, nrhs));
    hqr::pack_rhs_rows(atr, g.N, nrhs, g.N, G, g.M, g.NB, CT, s);
    TRY(hqr::trsmt_tiles(Af, g.M, g.N, g.NB, G, nrhs, s));
    // G = [h; d2], C = [d1 - h; d2]
    hqr::tile_rows(C, G, g.M, g.NB, CT, NT, MT, false, s);
    hqr::tile_rows(C, G, g.M, g.NB, CT, 0, NT, true, s);
    // x += R^-1 (d1 - h); r += Q [h; d2]
    TRY(hqr::trsm_tiles(Af, g.M, g.N, g.NB, C, nrhs, s));
    hqr::update_x(C, g.M, g.NB, g.N, nrhs, dX, ldx, true, s);
    TRY(cuda_rc(cudaGetLastError()));
    TRY(ormqr_n_cols(plan, Af, tau, G, CT, 1, s, nrhs));
    hqr::add_unpack(r, g.M, G, g.M, g.NB, nrhs, s);
    TRY(cuda_rc(cudaGetLastError()));
  }
  return ls_finish(plan, dA, dB, ldb, nrhs, dX, ldx, Res, nrm, resid, s);
}

int hqr_dgemm_tn(long N, int NB, const double* dA, const double* dB, double* dC, void* stream) {
  if (!dA || !dB || !dC || NB < 16 || NB % 16 || N <= 0 || N % NB) return HQR_ERR_INVALID;
  hqr::dgemm_tn_tiles(dA, dB, dC, N, N, NB, (cudaStream_t)stream);
  return cuda_rc(cudaGetLastError());
}

int hqr_make_identity(long M, long N, int NB, double* dQ, void* stream) {
  if (!dQ || NB <= 0 || M % NB || N % NB) return HQR_ERR_INVALID;
  hqr::make_identity(dQ, M, N, NB, true, (cudaStream_t)stream);
  return cuda_rc(cudaGetLastError());
}

int hqr_fill_uniform(long M, long N, int NB, uint64_t seed, double* dA, void* stream) {
  if (!dA || NB <= 0 || M % NB || N % NB) return HQR_ERR_INVALID;
  hqr::fill_uniform(dA, M, N, NB, seed, (cudaStream_t)stream);
  return cuda_rc(cudaGetLastError());
}

int hqr_frob2(long M, long N, int NB, const double* dX, const double* dY, double alpha,
              double* result, void* stream) {
  if (!dX || !result || NB <= 0 || M % NB || N % NB) return HQR_ERR_INVALID;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double)) != cudaSuccess) return HQR_ERR_NOMEM;
  cudaStream_t s = (cudaStream_t)stream;
  hqr::frob_diff(dX, dY, alpha, M, N, NB, d, s);
  int rc = cuda_rc(cudaMemcpyAsync(result, d, sizeof(double), cudaMemcpyDeviceToHost, s));
  if (rc == HQR_OK) rc = cuda_rc(cudaStreamSynchronize(s));
  cudaFree(d);
  return rc;
}

int hqr_tiles_to_colmajor(long M, long N, int NB, const double* dT, double* dCM, void* stream) {
  if (!dT || !dCM || NB <= 0 || M % NB || N % NB) return HQR_ERR_INVALID;
  hqr::tiles_to_colmajor(dT, dCM, M, N, NB, (cudaStream_t)stream);
  return cuda_rc(cudaGetLastError());
}

int hqr_colmajor_to_tiles(long M, long N, int NB, const double* dCM, double* dT, void* stream) {
  if (!dT || !dCM || NB <= 0 || M % NB || N % NB) return HQR_ERR_INVALID;
  hqr::colmajor_to_tiles(dCM, dT, M, N, NB, (cudaStream_t)stream);
  return cuda_rc(cudaGetLastError());
}

int hqr_colmajor_to_tiles_padded(long M, long N, long ld, int NB, const double* dCM, double* dT,
                                 void* stream) {
  if (!dT || !dCM || NB <= 0 || M <= 0 || N <= 0 || ld < M) return HQR_ERR_INVALID;
  hqr::colmajor_to_tiles_padded(dCM, ld, M, N, NB, dT, (cudaStream_t)stream);
  return cuda_rc(cudaGetLastError());
}

int hqr_tiles_to_colmajor_padded(long M, long N, long ld, int NB, const double* dT, double* dCM,
                                 void* stream) {
  if (!dT || !dCM || NB <= 0 || M <= 0 || N <= 0 || ld < M) return HQR_ERR_INVALID;
  hqr::tiles_to_colmajor_padded(dT, ld, M, N, NB, dCM, (cudaStream_t)stream);
  return cuda_rc(cudaGetLastError());
}

double hqr_fp64_peak_tflops(void* stream) {
  return hqr::measure_fp64_peak_tflops((cudaStream_t)stream);
}

int hqr_host_alloc(void** ptr, size_t bytes) {
  if (!ptr || bytes == 0) return HQR_ERR_INVALID;
  *ptr = nullptr;
  return cudaHostAlloc(ptr, bytes, cudaHostAllocDefault) == cudaSuccess ? HQR_OK : HQR_ERR_NOMEM;
}

int hqr_host_free(void* ptr) { return ptr ? cuda_rc(cudaFreeHost(ptr)) : HQR_OK; }

int hqr_dropin_phase_ms(double* out) {
  if (!out) return HQR_ERR_INVALID;
  std::lock_guard<std::mutex> lk(g_mu);
  for (int i = 0; i < 6; i++) out[i] = g_phase.ms[i];
  return HQR_OK;
}

double hqr_fp64_mma_peak_tflops(int shape, void* stream) {
  return hqr::measure_fp64_mma_peak_tflops(shape, (cudaStream_t)stream);
}

int hqr_zero_reflectors(long M, long N, int NB, double* dA, void* stream) {
  if (!dA || NB <= 0 || M % NB || N % NB) return HQR_ERR_INVALID;
  hqr::zero_reflectors(dA, M, N, NB, (cudaStream_t)stream);
  return cuda_rc(cudaGetLastError());
}

// ===========================================================================
// Drop-in entry points (Hybrid_tile_QR.h)
// ===========================================================================

static int do_tile_qr(mat_stat_t* st, double* A, double* TAU, int rank, int P, int ib) {
  TRY(check_status(st, rank, P));
  if (!A || !TAU) return HQR_ERR_INVALID;
  const long M = (long)st->my_mat_M, N = (long)st->my_mat_N;
  const int NB = (int)st->tile_M;
  hqr_plan* plan;
  TRY(stage_plan(M, N, NB, ib, &plan));
  cudaStream_t s;
  TRY(stage_stream(&s));
  double *dA, *dTAU;
  TRY(stage_reserve(0, (size_t)M * N, &dA));
  TRY(stage_reserve(1, tau_len(plan->g), &dTAU));
  phase_begin(s);
  TRY(h2d(dA, A, (size_t)M * N, s));
  TRY(h2d(dTAU, TAU, tau_len(plan->g), s));
  phase_mark(1, s);
  TRY(hqr_geqrf_async(plan, dA, dTAU, s));
  phase_mark(2, s);
  TRY(hqr_plan_status(plan, s));
  phase_mark(3, s);
  TRY(d2h(A, dA, (size_t)M * N, s));
  TRY(d2h(TAU, dTAU, tau_len(plan->g), s));
  phase_mark(4, s);
  TRY(cuda_rc(cudaStreamSynchronize(s)));
  phase_end();
  return HQR_OK;
}

void Hybrid_tile_QR(mat_stat_t* status, double* A, double* TAU, int my_rank, int Proc_num, int ib) {
  std::lock_guard<std::mutex> lk(g_mu);
  report("Hybrid_tile_QR", do_tile_qr(status, A, TAU, my_rank, Proc_num, ib));
}

void Hybrid_dgeqrf(mat_stat_t* status, double* A, double* TAU, int my_rank, int Proc_num) {
  std::lock_guard<std::mutex> lk(g_mu);
  report("Hybrid_dgeqrf",
         do_tile_qr(status, A, TAU, my_rank, Proc_num, status ? (int)status->tile_N : 0));
}

// Apply Q^T to a host array C (same grid) after staging RY, TAU; mode:
// 0 = make_Q (set diagonal, zero V), 1 = dorgqr (C := I first), 2 = dormqr.
static int do_apply(mat_stat_t* st, double* Q, double* RY, double* TAU, int rank, int P, int ib,
                    int mode) {
  TRY(check_status(st, rank, P));
  if (!Q || !RY || !TAU) return HQR_ERR_INVALID;
  const long M = (long)st->my_mat_M, N = (long)st->my_mat_N;
  const int NB = (int)st->tile_M;
  hqr_plan* plan;
  TRY(stage_plan(M, N, NB, ib > 0 ? ib : NB, &plan));
  cudaStream_t s;
  TRY(stage_stream(&s));
  double *dQ, *dRY, *dTAU;
  TRY(stage_reserve(0, (size_t)M * N, &dRY));
  TRY(stage_reserve(1, tau_len(plan->g), &dTAU));
  TRY(stage_reserve(2, (size_t)M * N, &dQ));
  phase_begin(s);
  TRY(h2d(dRY, RY, (size_t)M * N, s));
  TRY(h2d(dTAU, TAU, tau_len(plan->g), s));
  if (mode == 2 || (mode == 0 && plan->g.M != plan->g.N)) TRY(h2d(dQ, Q, (size_t)M * N, s));
  TRY(cuda_rc(cudaEventRecord(g_stage.h2d_done, s)));
  phase_mark(1, s);
  if (mode == 2) {
    bool rebuild;
    const hqr::OzWorkspace* oz = apply_operands(plan, false, false, &rebuild);
    TRY(hqr::launch_apply_qt(plan->g, &plan->ws, dRY, plan->dT, dTAU, dQ, plan->g.NT, rebuild,
                             g_timeout_ns, s, oz));
  } else {
    // make_Q (caller-zeroed Q, Hybrid_make_Q.c:91-95) and dorgqr (Q := I,
    // Hybrid_dorgqr.c:56) both produce Q^T of the factorization
    if (mode == 1) hqr::make_identity(dQ, M, N, NB, true, s);
    TRY(build_qt(plan, dQ, dRY, dTAU, false, s));   // the caller's reflectors: always prepared
  }
  phase_mark(2, s);
  if (mode == 0) {
    // R is the caller's RY with the reflectors zeroed: done on the host array
    // once the device has its copy, while the DAG runs (no copy back)
    TRY(cuda_rc(cudaEventSynchronize(g_stage.h2d_done)));
    host_zero_reflectors(RY, M, N, NB);
  }
  TRY(hqr_plan_status(plan, s));
  phase_mark(3, s);
  TRY(d2h(Q, dQ, (size_t)M * N, s));
  phase_mark(4, s);
  TRY(cuda_rc(cudaStreamSynchronize(s)));
  phase_end();
  return HQR_OK;
}

void Hybrid_make_Q(mat_stat_t* status, double* Q, double* RY, double* TAU, int my_rank,
                   int Proc_num, int ib) {
  std::lock_guard<std::mutex> lk(g_mu);
  report("Hybrid_make_Q", do_apply(status, Q, RY, TAU, my_rank, Proc_num, ib, 0));
}

void Hybrid_dorgqr(mat_stat_t* status, double* Q, double* RY, double* TAU, int my_rank,
                   int Proc_num) {
  std::lock_guard<std::mutex> lk(g_mu);
  report("Hybrid_dorgqr", do_apply(status, Q, RY, TAU, my_rank, Proc_num, 0, 1));
}

void Hybrid_dormqr(mat_stat_t* status, double* RY, double* TAU, double* C, int my_rank,
                   int Proc_num) {
  std::lock_guard<std::mutex> lk(g_mu);
  report("Hybrid_dormqr", do_apply(status, C, RY, TAU, my_rank, Proc_num, 0, 2));
}

static int do_simple(mat_stat_t* st, int rank, int P, int op, double* A, double* B, double* C) {
  TRY(check_status(st, rank, P));
  const long M = (long)st->my_mat_M, N = (long)st->my_mat_N;
  const int NB = (int)st->tile_M;
  if (op == 2 && M != N) return HQR_ERR_UNSUPPORTED;
  cudaStream_t s;
  TRY(stage_stream(&s));
  double *d0, *d1, *d2;
  TRY(stage_reserve(0, (size_t)M * N, &d0));
  if (op == 0) {            // identity
    if (!A) return HQR_ERR_INVALID;
    hqr::make_identity(d0, M, N, NB, true, s);
    TRY(d2h(A, d0, (size_t)M * N, s));
  } else if (op == 1) {     // zero reflectors
    if (!A) return HQR_ERR_INVALID;
    TRY(h2d(d0, A, (size_t)M * N, s));
    hqr::zero_reflectors(d0, M, N, NB, s);
    TRY(d2h(A, d0, (size_t)M * N, s));
  } else {                  // C = A^T B
    if (!A || !B || !C) return HQR_ERR_INVALID;
    if (NB % 16) return HQR_ERR_UNSUPPORTED;
    TRY(stage_reserve(1, (size_t)M * N, &d1));
    TRY(stage_reserve(2, (size_t)M * N, &d2));
    TRY(h2d(d0, A, (size_t)M * N, s));
    TRY(h2d(d1, B, (size_t)M * N, s));
    hqr::dgemm_tn_tiles(d0, d1, d2, M, N, NB, s);
    TRY(d2h(C, d2, (size_t)M * N, s));
  }
  TRY(cuda_rc(cudaGetLastError()));
  return cuda_rc(cudaStreamSynchronize(s));
}

void Hybrid_make_I(mat_stat_t* status, double* Id, int my_rank, int Proc_num) {
  std::lock_guard<std::mutex> lk(g_mu);
  report("Hybrid_make_I", do_simple(status, my_rank, Proc_num, 0, Id, nullptr, nullptr));
}

void Hybrid_remv_Y(mat_stat_t* status, double* RY, int my_rank, int Proc_num) {
  std::lock_guard<std::mutex> lk(g_mu);
  report("Hybrid_remv_Y", do_simple(status, my_rank, Proc_num, 1, RY, nullptr, nullptr));
}

void Hybrid_dgemm(mat_stat_t* status, double* A, double* B, double* C, int my_rank, int Proc_num) {
  std::lock_guard<std::mutex> lk(g_mu);
  report("Hybrid_dgemm", do_simple(status, my_rank, Proc_num, 2, A, B, C));
}

}  // extern "C"

// --- batches -------------------------------------------------------------------------
// Task tables of the two launch kinds (factorization, Q^T C): written on the
// host, uploaded through a pinned buffer when the pointers change, kept on
// the device for later calls (and graph replays) with the same pointers.
struct hqr_batch {
  int count = 0;
  std::vector<hqr::Geometry> g;
  std::vector<double*> T;    // per matrix, into dT
  // table order: the largest factorizations (longest task chains) first, so
  // that their first tasks are queued first and the launch ends with small ones
  std::vector<int> order;
  double* dT = nullptr;
  hqr::DagWorkspace ws;
  size_t smem = 0;
  int max_nrhs = 0;
  int ctas_per_sm = 1;   // executor CTAs per SM
  struct Table {
    std::vector<unsigned char> host;   // the descriptors last uploaded
    unsigned char* pinned = nullptr;
    void* dev = nullptr;
    cudaEvent_t uploaded = nullptr;
    int n_ids = 0, n_tasks = 0, nrhs = -1;
    bool valid = false;
  } tab[2];
};

namespace {
void free_batch(hqr_batch* b) {
  cudaFree(b->dT);
  hqr::dag_workspace_free(&b->ws);
  for (auto& t : b->tab) {
    cudaFreeHost(t.pinned);
    cudaFree(t.dev);
    if (t.uploaded) cudaEventDestroy(t.uploaded);
  }
  delete b;
}

// Make the device task table of launch kind `apply` describe these pointers.
int batch_table(hqr_batch* b, bool apply, double* const* dA, double* const* dTAU, double* const* dC,
                int nrhs, cudaStream_t s) {
  hqr_batch::Table& t = b->tab[apply ? 1 : 0];
  const size_t bytes = (size_t)b->count * hqr::mat_desc_bytes();
  std::vector<unsigned char> desc(bytes);
  int n_ids = 0, n_tasks = 0;
  TRY(hqr::batch_describe(apply, b->count, b->g.data(), b->order.data(), dA, b->T.data(), dTAU, dC, nrhs,
                          desc.data(), &n_ids, &n_tasks));
  if (t.valid && t.nrhs == nrhs && desc == t.host) return HQR_OK;   // the device copy is current
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  TRY(cuda_rc(cudaStreamIsCapturing(s, &cs)));
  if (cs != cudaStreamCaptureStatusNone) return HQR_ERR_UNSUPPORTED;   // upload outside a capture first
  TRY(cuda_rc(cudaEventSynchronize(t.uploaded)));   // the pinned buffer's previous copy is done
  memcpy(t.pinned, desc.data(), bytes);
  TRY(cuda_rc(cudaMemcpyAsync(t.dev, t.pinned, bytes, cudaMemcpyHostToDevice, s)));
  TRY(cuda_rc(cudaEventRecord(t.uploaded, s)));
  t.host.swap(desc);
  t.n_ids = n_ids;
  t.n_tasks = n_tasks;
  t.nrhs = nrhs;
  t.valid = true;
  return HQR_OK;
}
}  // namespace

extern "C" {

int hqr_batch_create(hqr_batch_t** batch, int count, const long* M, const long* N, const int* NB,
                     const int* IB, int max_nrhs, int ctas_per_sm) {
  if (!batch) return HQR_ERR_INVALID;
  *batch = nullptr;
  if (count <= 0 || !M || !N || !NB || !IB || max_nrhs < 0 || ctas_per_sm < 0 || ctas_per_sm > 2)
    return HQR_ERR_INVALID;
  hqr_batch* b = new hqr_batch();
  b->count = count;
  b->max_nrhs = max_nrhs;
  b->g.resize(count);
  size_t t_elems = 0;
  long long ids = 0, ids_apply = 0;
  // two CTAs per SM when every matrix's tiles fit half an SM's shared memory
  // (asked for, or by default when they all do)
  bool two = ctas_per_sm != 1;
  for (int i = 0; i < count && two; i++) {
    hqr::Geometry g;
    two = hqr::make_geometry(M[i], N[i], NB[i], IB[i], &g, hqr::batch_two_cta_smem()) == HQR_OK;
  }
  if (ctas_per_sm == 2 && !two) {
    free_batch(b);
    return HQR_ERR_UNSUPPORTED;
  }
  b->ctas_per_sm = two ? 2 : 1;
  for (int i = 0; i < count; i++) {
    const int rc = hqr::make_geometry(M[i], N[i], NB[i], IB[i], &b->g[i], two ? hqr::batch_two_cta_smem() : 0);
    if (rc != HQR_OK) {
      free_batch(b);
      return rc;
    }
    t_elems += (size_t)M[i] * N[i];
    b->smem = std::max(b->smem, b->g[i].smem_bytes);
    ids += hqr::batch_ids(false, b->g[i], 1);
    if (max_nrhs > 0) ids_apply += hqr::batch_ids(true, b->g[i], max_nrhs);
  }
  if (std::max(ids, ids_apply) > 0x3fffffffLL) {
    free_batch(b);
    return HQR_ERR_UNSUPPORTED;
  }
  const size_t bytes = (size_t)count * hqr::mat_desc_bytes();
  int rc = HQR_OK;
  if (cudaMalloc(&b->dT, t_elems * sizeof(double)) != cudaSuccess) rc = HQR_ERR_NOMEM;
  for (auto& t : b->tab) {
    if (rc != HQR_OK) break;
    if (cudaMallocHost(&t.pinned, bytes) != cudaSuccess || cudaMalloc(&t.dev, bytes) != cudaSuccess)
      rc = HQR_ERR_NOMEM;
    else if (cudaEventCreateWithFlags(&t.uploaded, cudaEventDisableTiming) != cudaSuccess)
      rc = HQR_ERR_CUDA;
  }
  if (rc == HQR_OK) rc = hqr::dag_workspace_reserve(&b->ws, (size_t)std::max(ids, ids_apply));
  if (rc != HQR_OK) {
    free_batch(b);
    return rc;
  }
  b->order.resize(count);
  for (int i = 0; i < count; i++) b->order[i] = i;
  auto work = [&](int i) {
    const hqr::Geometry& g = b->g[i];
    return (double)g.M * g.N * g.N - (double)g.N * g.N * g.N / 3.0;
  };
  std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) { return work(x) > work(y); });
  b->T.resize(count);
  size_t off = 0;
  for (int i = 0; i < count; i++) {
    b->T[i] = b->dT + off;
    off += (size_t)M[i] * N[i];
  }
  *batch = b;
  return HQR_OK;
}

int hqr_batch_destroy(hqr_batch_t* batch) {
  if (!batch) return HQR_ERR_INVALID;
  free_batch(batch);
  return HQR_OK;
}

int hqr_batch_geqrf_async(hqr_batch_t* b, double* const* dA, double* const* dTAU, void* stream) {
  if (!b || !dA || !dTAU) return HQR_ERR_INVALID;
  for (int i = 0; i < b->count; i++)
    if (!dA[i] || !dTAU[i]) return HQR_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  TRY(batch_table(b, false, dA, dTAU, dA, 0, s));
  const hqr_batch::Table& t = b->tab[0];
  return hqr::launch_batch(false, b->count, t.dev, t.n_ids, t.n_tasks, b->smem, b->ctas_per_sm, &b->ws, g_timeout_ns, s);
}

int hqr_batch_geqrf(hqr_batch_t* b, double* const* dA, double* const* dTAU, void* stream) {
  TRY(hqr_batch_geqrf_async(b, dA, dTAU, stream));
  return hqr_batch_status(b, stream);
}

int hqr_batch_ormqr_t_async(hqr_batch_t* b, double* const* dA, double* const* dTAU, double* const* dC,
                            int nrhs, void* stream) {
  if (!b || !dA || !dTAU || !dC || nrhs <= 0 || nrhs > b->max_nrhs) return HQR_ERR_INVALID;
  for (int i = 0; i < b->count; i++)
    if (!dA[i] || !dTAU[i] || !dC[i]) return HQR_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  TRY(batch_table(b, true, dA, dTAU, dC, nrhs, s));
  const hqr_batch::Table& t = b->tab[1];
  return hqr::launch_batch(true, b->count, t.dev, t.n_ids, t.n_tasks, b->smem, b->ctas_per_sm, &b->ws, g_timeout_ns, s);
}

int hqr_batch_ormqr_t(hqr_batch_t* b, double* const* dA, double* const* dTAU, double* const* dC, int nrhs,
                      void* stream) {
  TRY(hqr_batch_ormqr_t_async(b, dA, dTAU, dC, nrhs, stream));
  return hqr_batch_status(b, stream);
}

int hqr_batch_ctas_per_sm(hqr_batch_t* b) { return b ? b->ctas_per_sm : 0; }

int hqr_batch_status(hqr_batch_t* b, void* stream) {
  if (!b) return HQR_ERR_INVALID;
  return hqr::dag_status(&b->ws, (cudaStream_t)stream);
}

int hqr_batch_stats(hqr_batch_t* b, hqr_stats_t* out, void* stream) {
  if (!b || !out) return HQR_ERR_INVALID;
  unsigned long long v[14];
  TRY(hqr::dag_stats(&b->ws, v, (cudaStream_t)stream));
  for (int t = 0; t < 7; t++) {
    out->count[t] = v[2 * t];
    out->cycles[t] = v[2 * t + 1];
  }
  return HQR_OK;
}

}  // extern "C"
