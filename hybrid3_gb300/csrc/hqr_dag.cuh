// hqr_dag.cuh -- the device-resident tile DAG: dependency counters, ready
// queues and the persistent executor kernel.
//
// This replaces, on the GPU, the reference's OpenMP task machinery:
//   * prog_table (Hybrid_tile_QR.c:23,36-40,515-580): one byte per task
//     (i,j,k) whose MEM/LIN/YTM bits become ready at 0x7.  Here each task owns
//     an int counter initialised to its number of unmet inputs and a task is
//     ready when an atomic decrement brings it to zero:
//       MEM  -- the tile was updated by the previous step's SSRFB,
//       LIN  -- the previous task of the same column chain is done,
//       YTM  -- the panel reflector (Y, T) the update needs is available.
//   * the TileSch FIFO (TileSch.c:10-61) under omp critical becomes two
//     lock-free FIFOs in global memory, one for the critical path (panel tasks
//     and the next panel column's updates) and one for the rest.  Each queue
//     has room for every task (each task is pushed exactly once), so a push
//     never waits.
//   * the Y/T ring glob_YT with its tickets (Hybrid_tile_QR.c:379-390) is not
//     needed: V stays in place in A and every panel tile's T is kept in HBM.
//   * the worker loop (Hybrid_tile_QR.c:905-1461) becomes a persistent kernel
//     with one CTA per SM; thread 0 pops, the CTA runs the task, thread 0
//     releases its dependents.
//
// LARFB and SSRFB tasks are split into NC column blocks (the columns of a
// trailing tile are independent), which multiplies the parallelism of a step
// by NC.  The factorization's panel tasks are split into their w-column inner
// blocks: block b of the TSQRT of tile k needs block b of tile k-1's panel
// (the last writer of R's rows [b w, (b+1) w)) and block b-1 of its own tile,
// so the TS chain down a panel column runs as a wavefront, MT + NB/w block
// steps deep instead of MT NB/w.  Every wait is bounded in time: when a wait runs out the kernel sets
// an error bit and every CTA returns, so a broken DAG never hangs the GPU.
#pragma once
#include <type_traits>
#include "hqr_oztasks.cuh"
#include "hqr_tile_fp64.cuh"

namespace hqr {

enum DagMode : int {
  kModeFactor = 0,    // Hybrid_tile_QR: GEQRT/TSQRT panels + LARFB/SSRFB updates of A
  kModeApplyQt = 1,   // C <- Q^T C: T-build panels + LARFB/SSRFB updates of C
  // Q <- Q_0 Q_1 ... Q_{steps-1} C for C = I (square): the panel columns from
  // the last to the first, each panel tile's reflector H (not H^T), tile rows
  // from the bottom up; step i touches tile columns j >= i only (columns j < i
  // are still unit vectors in rows >= i), 2/3 of the updates of kModeApplyQt.
  kModeBuildQ = 2,
  // C <- Q C = H_0 H_1 ... H_{steps-1} C for a general C of CT tile columns
  // (LAPACK dormqr 'L','N'): kModeBuildQ's order and arithmetic (H, not H^T)
  // on every tile column.
  kModeApplyQ = 3,
};
// The modes that apply H itself (not H^T).
__host__ __device__ __forceinline__ bool applies_h(int mode) { return mode == kModeBuildQ || mode == kModeApplyQ; }

// With split precision (DagParams::oz) the update tasks run OZAPPLY and every
// panel tile gets an OZPREP task (in the factorization it follows the
// GEQRT/TSQRT; in the Q^T application it replaces the T-build).
enum TaskType : int {
  kGEQRT = 0, kTSQRT = 1, kLARFB = 2, kSSRFB = 3, kTBUILD = 4, kOZPREP = 5, kNumTypes = 6,
  // the merges of a domain tree (counted with TSQRT, OZPREP and SSRFB)
  kTTQRT = 6, kTTPREP = 7, kTTMQR = 8
};
__host__ __device__ __forceinline__ int stat_slot(int type) {
  return type == kTTQRT ? kTSQRT : type == kTTPREP ? kOZPREP : type == kTTMQR ? kSSRFB : type;
}
// Statistics slots: one per task type, then the scheduler's own time (thread
// 0 of each CTA: popping the next task and releasing the dependents).
constexpr int kStatSched = kNumTypes, kNumStats = kNumTypes + 1;

// Control words of the scheduler (one cache line each is not needed: the
// counters are touched once per task).
enum Ctl : int { kHiHead = 0, kHiTail = 1, kLoHead = 2, kLoTail = 3, kDone = 4, kErr = 5, kCtlWords = 8 };

// One matrix of a batch (batched DAG): its geometry, task-id range and arrays.
struct MatDesc {
  int MT, NT, CT, NC, steps, J, nblk;
  TileShape sh;
  SmemPlan sp;
  double *A, *T, *TAU, *C;
  int id_base;   // first global task id of this matrix
  int id_end;    // one past its last (the next matrix's id_base)
};

struct DagParams {
  int mode;
  int MT, NT, CT, NC, steps, J;   // J = tile columns spanned by update ids
  int nblk;                        // panel inner blocks per panel task id (factorization: NB / w)
  // Domain tree (tree > 0): at step i the tile rows i.. are cut into domains of
  // `tree` tiles; each domain runs the flat TS chain on its own top tile, then
  // the domain tops' R are merged into R(i, i) one after the other by TT
  // kernels (CORE_dttqrt / CORE_dttmqr).  tree = 0: one domain (flat tree).
  int tree, dmax;                  // domain size, maximum number of domains
  int skip_panels;                 // 1: the panel tasks' T / slices come from the factorization
  double* T2;                      // T of each merge, compact: tile (i * dmax + d)
  double* TAU2;                    // TAU of each merge, compact: (i * dmax + d) * NB
  uint8_t* slices2;                // split: the merges' prepared operands, compact
  int* sexp2;
  // Batch (n_mats > 0): the task ids of matrix m are [mats[m].id_base, + its
  // count); counters and queues hold global ids, and every task runs with its
  // matrix's fields copied over these (id_base included).
  int id_base;
  int n_mats;
  const MatDesc* mats;
  TileShape sh;
  SmemPlan sp;
  double* A;        // factored matrix: R above, V below the diagonal
  double* T;        // T tiles (same tile layout as A)
  double* TAU;
  double* C;        // target of the update tasks (A itself when factoring)
  int* cnt;         // dependency counters, one per task id
  // Factorization with the flat tree (ts_split): a panel block (GEQRT or
  // TSQRT inner block b of tile k at step i) releases the same block of the
  // tile below once its reflectors are stored, and the next block of its
  // own tile once the next block's w columns are updated; tsflag[its id]
  // is set when its whole trailing update is done, which the later blocks
  // that share those columns or R's rows wait for (bounded) before theirs.
  int ts_split;
  int ts_split_from;   // the first step whose panel blocks use the phases
  int* tsflag;
  int* qhi;         // ready FIFOs, capacity n_ids each
  int* qlo;
  unsigned* ctl;
  int n_ids;        // size of the task-id space
  int n_tasks;      // number of real tasks
  long long timeout_ns;
  unsigned long long* stats;   // [type][0] = count, [type][1] = SM cycles
  // split precision
  int oz;           // 1: OZPREP/OZAPPLY tasks (NC * oz_cpt = NB / 64)
  int oz_cpt;       // 64-column chunks one OZAPPLY task updates, one after the other
  // Q applications: columns of C that hold data (0: all); the column blocks
  // from there on are zero, stay zero, and their updates are skipped
  long long c_cols;
  int oz_groups;    // t-groups of the split updates (8 or 4; host side: picks the kernel)
  int oz_p32;       // 1: FP32 panel arithmetic (host side: picks the kernel)
  int prep;         // 1: separate OZPREP ids after the panel ids (factorization)
  uint8_t* slices;  // sliced left operands, one block per panel tile
  int* sexp;        // their row exponents (oz::kSlots * NB ints per panel tile)
};

constexpr int kNever = 0x3fffffff;

// Release / acquire fence at GPU scope.  A task's results reach its
// dependents by message passing: every thread fences its writes, the CTA
// synchronises, thread 0 decrements the dependents' counters; the CTA that
// takes a dependent fences after observing its counter reach zero.  That
// needs acquire-release ordering only, not the sequentially consistent fence
// of __threadfence().
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// --- domains -------------------------------------------------------------------
__host__ __device__ __forceinline__ int dom_size(const DagParams& p) { return p.tree > 0 ? p.tree : p.MT; }
__host__ __device__ __forceinline__ int dom_of(const DagParams& p, int i, int k) { return (k - i) / dom_size(p); }
__host__ __device__ __forceinline__ int dom_top(const DagParams& p, int i, int d) { return i + d * dom_size(p); }
__host__ __device__ __forceinline__ int dom_end(const DagParams& p, int i, int d) {
  const int e = i + (d + 1) * dom_size(p);
  return e < p.MT ? e : p.MT;
}
__host__ __device__ __forceinline__ int n_domains(const DagParams& p, int i) {
  return p.tree > 0 ? (p.MT - i + p.tree - 1) / p.tree : 1;
}
__host__ __device__ __forceinline__ bool is_top(const DagParams& p, int i, int k) {
  return (k - i) % dom_size(p) == 0;
}

// --- task ids ----------------------------------------------------------------
//   panel  (i, k, b)     : (i*MT + k)*nblk + b                   (k >= i)
//   prep   (i, k)        : P0 + i*MT + k   (factorization with split precision)
//   update (i, j, k, c)  : U0 + ((i*J + j)*MT + k)*NC + c        (k >= i)
//   merge  (i, d, b)     : M0 + (i*dmax + d)*nblk + b            (1 <= d < domains)
//   merge prep (i, d)    : Q0 + i*dmax + d     (split precision)
//   merge update (i, j, d, c): X0 + ((i*J + j)*dmax + d)*NC + c
__host__ __device__ __forceinline__ int panel_id(const DagParams& p, int i, int k, int b = 0) {
  return (i * p.MT + k) * p.nblk + b;
}
__host__ __device__ __forceinline__ int panel_end(const DagParams& p) {
  return p.steps * p.MT * p.nblk;
}
__host__ __device__ __forceinline__ int prep_id(const DagParams& p, int i, int k) {
  return panel_end(p) + i * p.MT + k;
}
__host__ __device__ __forceinline__ int update_base(const DagParams& p) {
  return panel_end(p) + (p.prep ? p.steps * p.MT : 0);
}
__host__ __device__ __forceinline__ int update_id(const DagParams& p, int i, int j, int k, int c) {
  return update_base(p) + ((i * p.J + j) * p.MT + k) * p.NC + c;
}
__host__ __device__ __forceinline__ int update_end(const DagParams& p) {
  return update_base(p) + p.steps * p.J * p.MT * p.NC;
}
__host__ __device__ __forceinline__ int merge_id(const DagParams& p, int i, int d, int b) {
  return update_end(p) + (i * p.dmax + d) * p.nblk + b;
}
__host__ __device__ __forceinline__ int ttprep_base(const DagParams& p) {
  return update_end(p) + p.steps * p.dmax * p.nblk;
}
__host__ __device__ __forceinline__ int ttprep_id(const DagParams& p, int i, int d) {
  return ttprep_base(p) + i * p.dmax + d;
}
__host__ __device__ __forceinline__ int ttmqr_base(const DagParams& p) {
  return ttprep_base(p) + (p.prep ? p.steps * p.dmax : 0);
}
__host__ __device__ __forceinline__ int ttmqr_id(const DagParams& p, int i, int j, int d, int c) {
  return ttmqr_base(p) + ((i * p.J + j) * p.dmax + d) * p.NC + c;
}
__host__ __device__ __forceinline__ int id_end(const DagParams& p) {
  return ttmqr_base(p) + p.steps * p.J * p.dmax * p.NC;
}
// Compact index of merge (i, d) into T2 / TAU2 / slices2.
__host__ __device__ __forceinline__ size_t merge_slot(const DagParams& p, int i, int d) {
  return (size_t)i * p.dmax + d;
}
// Compact index of panel tile (k, i), k >= i, into the slice store.
__host__ __device__ __forceinline__ size_t panel_slot(int MT, int i, int k) {
  return (size_t)i * MT - (size_t)i * (i - 1) / 2 + (size_t)(k - i);
}

struct TaskDesc {
  int type, i, j, k, c;   // c: column block of an update, inner block of a panel task
};

__device__ __forceinline__ TaskDesc decode(const DagParams& p, int id) {
  TaskDesc t;
  const int P0 = panel_end(p);
  const int U0 = update_base(p);
  if (id < P0) {
    const int tile = id / p.nblk;
    t.i = tile / p.MT;
    t.k = tile % p.MT;
    t.j = t.i;
    t.c = id % p.nblk;
    if (p.mode == kModeFactor)
      t.type = is_top(p, t.i, t.k) ? kGEQRT : kTSQRT;
    else
      t.type = p.oz ? kOZPREP : kTBUILD;
  } else if (id < U0) {
    t.i = (id - P0) / p.MT;
    t.k = (id - P0) % p.MT;
    t.j = t.i;
    t.c = 0;
    t.type = kOZPREP;
  } else if (id < update_end(p)) {
    int u = id - U0;
    t.c = u % p.NC; u /= p.NC;
    t.k = u % p.MT; u /= p.MT;
    t.j = u % p.J;
    t.i = u / p.J;
    t.type = is_top(p, t.i, t.k) ? kLARFB : kSSRFB;
  } else if (id < ttprep_base(p)) {
    int u = id - update_end(p);
    t.c = u % p.nblk; u /= p.nblk;
    const int d = u % p.dmax;
    t.i = u / p.dmax;
    t.j = t.i;
    t.k = dom_top(p, t.i, d);
    t.type = kTTQRT;
  } else if (id < ttmqr_base(p)) {
    const int u = id - ttprep_base(p);
    const int d = u % p.dmax;
    t.i = u / p.dmax;
    t.j = t.i;
    t.k = dom_top(p, t.i, d);
    t.c = 0;
    t.type = kTTPREP;
  } else {
    int u = id - ttmqr_base(p);
    t.c = u % p.NC; u /= p.NC;
    const int d = u % p.dmax; u /= p.dmax;
    t.j = u % p.J;
    t.i = u / p.J;
    t.k = dom_top(p, t.i, d);
    t.type = kTTMQR;
  }
  return t;
}

__device__ __forceinline__ bool update_valid(const DagParams& p, int i, int j) {
  if (p.mode == kModeFactor) return j > i && j < p.NT;
  if (p.mode == kModeBuildQ) return j >= i && j < p.CT;
  return j < p.CT;
}

__device__ __forceinline__ bool is_high_priority(const DagParams& p, int id) {
  const TaskDesc t = decode(p, id);
  if (t.type == kGEQRT || t.type == kTSQRT || t.type == kTBUILD || t.type == kOZPREP ||
      t.type == kTTQRT || t.type == kTTPREP)
    return true;
  return p.mode == kModeFactor && t.j == t.i + 1;   // look-ahead: next panel column
}

// --- queues -------------------------------------------------------------------
// Queue global task id gid (queues hold global ids).
__device__ __forceinline__ void push_queue(const DagParams& p, int gid, bool hi) {
  int* q = hi ? p.qhi : p.qlo;
  const unsigned slot = atomicAdd(p.ctl + (hi ? kHiTail : kLoTail), 1u);
  if ((int)slot < p.n_ids) {
    atomicExch(q + slot, gid);
  } else {
    atomicOr((int*)(p.ctl + kErr), kErrBadTask);
  }
}
__device__ __forceinline__ void push_ready(const DagParams& p, int id) {
  push_queue(p, p.id_base + id, is_high_priority(p, id));
}

// One input of task `id` is available (the releasing task's writes were fenced
// before).  A task that becomes ready is queued, or, when `keep` is given and
// still empty and the task is not on the high-priority queue, handed back to
// the caller to run next (a continuation: no queue round trip).
__device__ __forceinline__ void release(const DagParams& p, int id, int* keep = nullptr) {
  if (atomicSub(p.cnt + p.id_base + id, 1) == 1) {
    if (keep && *keep < 0 && !is_high_priority(p, id))
      *keep = p.id_base + id;
    else
      push_ready(p, id);
  }
}

// release() for up to 4 dependents at once: the counter decrements go out
// back to back, so their round trips to L2 overlap, then the ones that became
// ready are queued or kept (the first low-priority one, as release() keeps).
// True when one of them went to the high-priority queue.
__device__ __forceinline__ bool release_n(const DagParams& p, const int (&ids)[4], int n, int* keep) {
  bool hi = false;
  int old[4];
#pragma unroll
  for (int q = 0; q < 4; q++)
    if (q < n) old[q] = atomicSub(p.cnt + p.id_base + ids[q], 1);
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (q < n && old[q] == 1) {
      const bool h = is_high_priority(p, ids[q]);
      hi = hi || h;
      if (keep && *keep < 0 && !h)
        *keep = p.id_base + ids[q];
      else
        push_ready(p, ids[q]);
    }
  }
  return hi;
}

// Wait (bounded) until slot of queue q has been written; returns the id or -1.
__device__ int wait_slot(const DagParams& p, int* q, unsigned slot) {
  const uint64_t t0 = global_ns();
  for (;;) {
    const int v = *((volatile int*)(q + slot));
    if (v >= 0) return v;
    if ((long long)(global_ns() - t0) > p.timeout_ns) {
      atomicOr((int*)(p.ctl + kErr), kErrTimeout);
      return -1;
    }
    __nanosleep(64);
  }
}

__device__ __forceinline__ int try_claim(const DagParams& p, int* q, int head, int tail) {
  volatile unsigned* ctl = p.ctl;
  unsigned h = ctl[head];
  while (h < ctl[tail]) {
    const unsigned prev = atomicCAS(p.ctl + head, h, h + 1);
    if (prev == h) return wait_slot(p, q, h);
    h = prev;
  }
  return -2;   // nothing to claim
}

// Thread 0: next task id, or -1 when the DAG is done or failed.
__device__ int pop_task(const DagParams& p) {
  volatile unsigned* ctl = p.ctl;
  uint64_t t0 = global_ns();
  unsigned ns = 32;
  for (;;) {
    if (ctl[kErr] != 0u) return -1;
    if ((int)ctl[kDone] >= p.n_tasks) return -1;
    int id = try_claim(p, p.qhi, kHiHead, kHiTail);
    if (id == -2) id = try_claim(p, p.qlo, kLoHead, kLoTail);
    if (id >= 0) {
      fence_acq_rel_gpu();   // acquire: the producers' tile writes are visible
      return id;
    }
    if (id == -1) return -1;
    if ((long long)(global_ns() - t0) > p.timeout_ns) {
      atomicOr((int*)(p.ctl + kErr), kErrTimeout);
      return -1;
    }
    __nanosleep(ns);
    if (ns < 1024) ns <<= 1;
  }
}

// --- dependency initialisation (one thread per id) --------------------------------
__device__ int init_deps(const DagParams& p, int id) {
  int deps = kNever;
  const int P0 = panel_end(p);
  const int U0 = update_base(p);
  const int U1 = update_end(p);
  if (id < P0) {
    const int tile = id / p.nblk, b = id % p.nblk;
    const int i = tile / p.MT, k = tile % p.MT;
    if (k >= i && !p.skip_panels) {
      // block 0: the previous step's update of the tile (NC column blocks);
      // block b > 0: block b - 1 of the same tile; a TSQRT block also waits
      // for the same block of the tile above (its domain top's rows of R)
      if (p.mode == kModeFactor)
        deps = (b == 0 ? (i > 0 ? p.NC : 0) : 1) + (is_top(p, i, k) ? 0 : 1);
      else
        deps = 0;
    }
  } else if (id < U0) {
    const int i = (id - P0) / p.MT, k = (id - P0) % p.MT;
    if (k >= i) deps = 1;   // its panel task
  } else if (id < U1) {
    int u = id - U0;
    u /= p.NC;
    const int k = u % p.MT; u /= p.MT;
    const int j = u % p.J;
    const int i = u / p.J;
    if (k >= i && i < p.steps && update_valid(p, i, j)) {
      if (applies_h(p.mode))   // panel (unless given) + chain from the tile below + step i+1's write of (k, j)
        deps = (p.skip_panels ? 0 : 1) + (k < p.MT - 1 ? 1 : 0) +
               ((k > i && (j > i || p.mode == kModeApplyQ) && i + 1 < p.steps) ? 1 : 0);
      else   // panel (unless given) + the chain above in the domain + the previous step's write
        deps = (p.skip_panels ? 0 : 1) + (is_top(p, i, k) ? 0 : 1) + (i > 0 ? 1 : 0);
    }
  } else if (id < ttprep_base(p)) {
    // merge block b of domain d: block b - 1, domain d's chain (its last tile,
    // block b), the previous merge's block b (domain 0's chain for d = 1)
    int u = id - U1;
    const int b = u % p.nblk; u /= p.nblk;
    const int d = u % p.dmax, i = u / p.dmax;
    if (i < p.steps && d >= 1 && d < n_domains(p, i) && !p.skip_panels) deps = (b > 0 ? 1 : 0) + 2;
  } else if (id < ttmqr_base(p)) {
    const int u = id - ttprep_base(p);
    const int d = u % p.dmax, i = u / p.dmax;
    if (i < p.steps && d >= 1 && d < n_domains(p, i) && !p.skip_panels) deps = 1;
  } else {
    // merge update: the merge (unless given), domain d's chain on column j,
    // the previous merge update (domain 0's chain for d = 1)
    int u = id - ttmqr_base(p);
    u /= p.NC;
    const int d = u % p.dmax; u /= p.dmax;
    const int j = u % p.J, i = u / p.J;
    if (i < p.steps && d >= 1 && d < n_domains(p, i) && update_valid(p, i, j))
      deps = (p.skip_panels ? 0 : 1) + 2;
  }
  return deps;
}

__global__ void dag_init_kernel(DagParams p) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= p.n_ids) return;
  p.qhi[id] = -1;
  p.qlo[id] = -1;
  p.cnt[id] = init_deps(p, id);
  if (p.ts_split && id < panel_end(p)) p.tsflag[id] = 0;
}

__global__ void dag_seed_kernel(DagParams p) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= p.n_ids) return;
  if (p.cnt[id] == 0) push_ready(p, id);
}

// --- batches ---------------------------------------------------------------------
__device__ __forceinline__ void apply_mat(DagParams& q, const MatDesc& d) {
  q.MT = d.MT;
  q.NT = d.NT;
  q.CT = d.CT;
  q.NC = d.NC;
  q.steps = d.steps;
  q.J = d.J;
  q.nblk = d.nblk;
  q.sh = d.sh;
  q.sp = d.sp;
  q.A = d.A;
  q.T = d.T;
  q.TAU = d.TAU;
  q.C = d.C;
  q.id_base = d.id_base;
}
// Warp 0: the matrix that global task id g belongs to (ids are laid out by
// matrix), a 32-way search: three dependent loads for 4096 matrices.
__device__ __forceinline__ int find_mat_warp(const DagParams& p, int g) {
  const int lane = threadIdx.x & 31;
  int lo = 0, hi = p.n_mats;   // mats[lo].id_base <= g < mats[hi].id_base
  while (hi - lo > 1) {
    const int step = (hi - lo + 31) >> 5;
    const int idx = lo + lane * step;
    const bool le = idx < hi && __ldg(&p.mats[idx].id_base) <= g;
    const unsigned b = __ballot_sync(0xffffffffu, le);
    const int nlo = lo + (31 - __clz(b)) * step;
    hi = min(hi, nlo + step);
    lo = nlo;
  }
  return lo;
}
// Shared state of a batched executor CTA: the current task's matrix fields.
template <bool BATCH> struct BatchLocal {
  DagParams lp;
  int end;   // one past lp's task ids (0: none loaded yet)
};
template <> struct BatchLocal<false> {};
__device__ __forceinline__ const DagParams& local_params(const DagParams& p, BatchLocal<false>&) { return p; }
__device__ __forceinline__ const DagParams& local_params(const DagParams&, BatchLocal<true>& b) { return b.lp; }
__device__ __forceinline__ void init_local(BatchLocal<false>&) {}
__device__ __forceinline__ void init_local(BatchLocal<true>& b) {
  if (threadIdx.x == 0) {
    b.lp.id_base = 0;
    b.end = 0;
  }
}
// All threads: make b.lp the fields of the matrix that owns gid.
__device__ __forceinline__ void load_local(const DagParams& p, BatchLocal<false>&, int) {}
__device__ __forceinline__ void load_local(const DagParams& p, BatchLocal<true>& b, int gid) {
  if (threadIdx.x < 32) {
    const bool have = gid >= b.lp.id_base && gid < b.end;
    __syncwarp();
    if (!have) {
      const int m = find_mat_warp(p, gid);
      if (threadIdx.x == 0) {
        b.lp = p;
        apply_mat(b.lp, p.mats[m]);
        b.end = p.mats[m].id_end;
      }
    }
  }
  __syncthreads();
}
// One block per matrix: its ids' counters and queue slots, then (second
// kernel) the ready ones pushed.
__global__ void dag_init_batch_kernel(DagParams p) {
  __shared__ DagParams q;
  if (threadIdx.x == 0) {
    q = p;
    apply_mat(q, p.mats[blockIdx.x]);
  }
  __syncthreads();
  const int end = (blockIdx.x + 1 < p.n_mats) ? p.mats[blockIdx.x + 1].id_base : p.n_ids;
  for (int lid = threadIdx.x; q.id_base + lid < end; lid += blockDim.x) {
    const int g = q.id_base + lid;
    p.qhi[g] = -1;
    p.qlo[g] = -1;
    p.cnt[g] = init_deps(q, lid);
  }
}
__global__ void dag_seed_batch_kernel(DagParams p) {
  __shared__ DagParams q;
  if (threadIdx.x == 0) {
    q = p;
    apply_mat(q, p.mats[blockIdx.x]);
  }
  __syncthreads();
  const int end = (blockIdx.x + 1 < p.n_mats) ? p.mats[blockIdx.x + 1].id_base : p.n_ids;
  for (int lid = threadIdx.x; q.id_base + lid < end; lid += blockDim.x)
    if (p.cnt[q.id_base + lid] == 0) push_ready(q, lid);
}

// --- releases after a task ---------------------------------------------------------
// Step i has finished tile (k, j): its next consumer is step i + 1's update
// (or, in the factorization, its panel task when j = i + 1); -1 at the last step.
__device__ __forceinline__ int mem_consumer(const DagParams& p, int i, int j, int k, int c) {
  if (i + 1 >= p.steps) return -1;
  if (p.mode == kModeFactor && j == i + 1) return panel_id(p, i + 1, k, 0);
  return update_id(p, i + 1, j, k, c);
}
__device__ __forceinline__ void push_id(int (&ids)[4], int& n, int id) {
  if (id >= 0) ids[n++] = id;
}

// keep: receives at most one ready low-priority dependent to run next.
// Returns true when a high-priority task may have become ready (panel-type
// tasks always report so).
__device__ bool release_dependents(const DagParams& p, const TaskDesc& t, int* keep) {
  if (t.type == kGEQRT || t.type == kTSQRT || t.type == kTBUILD || t.type == kOZPREP) {
    const bool feeds_prep = (t.type == kGEQRT || t.type == kTSQRT) && p.prep;
    const bool panel = (t.type == kGEQRT || t.type == kTSQRT);
    if (panel) {
      // the next inner block of this tile; the same block of the tile below in
      // the domain, or, from a domain's last tile, of the domain's merge
      const int d = dom_of(p, t.i, t.k);
      if (!p.ts_split || t.i < p.ts_split_from) {   // (else the task's phases released these)
        if (t.c + 1 < p.nblk) release(p, panel_id(p, t.i, t.k, t.c + 1));
        if (t.k + 1 < dom_end(p, t.i, d))
          release(p, panel_id(p, t.i, t.k + 1, t.c));
        else if (n_domains(p, t.i) > 1)
          release(p, merge_id(p, t.i, d >= 1 ? d : 1, t.c));
      }
      if (t.c + 1 < p.nblk) return true;   // the tile's V, T, TAU are complete after its last block
    }
    if (feeds_prep) {
      release(p, prep_id(p, t.i, t.k));
    } else {
      const int j0 = (p.mode == kModeFactor) ? t.i + 1 : (p.mode == kModeBuildQ) ? t.i : 0;
      const int j1 = (p.mode == kModeFactor) ? p.NT : p.CT;
      for (int j = j0; j < j1; j++)
        for (int c = 0; c < p.NC; c++) release(p, update_id(p, t.i, j, t.k, c));
    }
    return true;
  }
  if (t.type == kTTQRT || t.type == kTTPREP) {
    const int d = dom_of(p, t.i, t.k);
    if (t.type == kTTQRT) {
      if (t.c + 1 < p.nblk) release(p, merge_id(p, t.i, d, t.c + 1));
      if (d + 1 < n_domains(p, t.i)) release(p, merge_id(p, t.i, d + 1, t.c));
      if (t.c + 1 < p.nblk) return true;
      if (p.prep) {
        release(p, ttprep_id(p, t.i, d));
        return true;
      }
    }
    for (int j = t.i + 1; j < p.NT; j++)
      for (int c = 0; c < p.NC; c++) release(p, ttmqr_id(p, t.i, j, d, c));
    return true;
  }
  int ids[4], n = 0;
  if (t.type == kTTMQR) {
    const int d = dom_of(p, t.i, t.k);
    if (d + 1 < n_domains(p, t.i)) push_id(ids, n, ttmqr_id(p, t.i, t.j, d + 1, t.c));
    push_id(ids, n, mem_consumer(p, t.i, t.j, t.k, t.c));   // the domain top's tile row is final
  } else if (applies_h(p.mode)) {
    // the chain runs from the bottom tile up to the LARFB; the step before
    // (i - 1) next writes tile (k, j), which this task wrote last
    if (t.k - 1 >= t.i) push_id(ids, n, update_id(p, t.i, t.j, t.k - 1, t.c));
    if (t.i >= 1) push_id(ids, n, update_id(p, t.i - 1, t.j, t.k, t.c));
  } else {
    // LARFB / SSRFB: LIN to the next task of this domain's column chain, or
    // from the domain's last tile to its merge update
    const int d = dom_of(p, t.i, t.k);
    if (t.k + 1 < dom_end(p, t.i, d))
      push_id(ids, n, update_id(p, t.i, t.j, t.k + 1, t.c));
    else if (n_domains(p, t.i) > 1)
      push_id(ids, n, ttmqr_id(p, t.i, t.j, d >= 1 ? d : 1, t.c));
    // MEM: an SSRFB's lower tile is final for this step (a LARFB's tile row
    // is final, or, at a domain top, finished by the merge update)
    if (t.type == kSSRFB) push_id(ids, n, mem_consumer(p, t.i, t.j, t.k, t.c));
  }
  return release_n(p, ids, n, keep);
}

// --- T build for the Q^T application (diagonal w x w blocks from V, TAU) -------
__device__ void task_tbuild(const double* V, const double* tau_g, double* T, bool unit,
                            const TileShape& sh, double* smem, const SmemPlan& sp) {
  const int NB = sh.NB, w = sh.w;
  double* sP = smem + sp.off_c1;
  double* sTau = smem + sp.off_tau;
  double* sG = smem + sp.off_g;
  double* sTb = smem + sp.off_t;
  for (int i0 = 0; i0 < NB; i0 += w) {
    const int m = unit ? NB - i0 : NB;
    const double* src = unit ? V + i0 + (size_t)i0 * NB : V + (size_t)i0 * NB;
    __syncthreads();
    load_block(sP, NB, src, NB, m, w);
    for (int e = threadIdx.x; e < w; e += kThreads) sTau[e] = ldg_cg(tau_g + i0 + e);
    __syncthreads();
    build_t_block(sP, NB, m, w, unit, sTau, sG, sTb);
    store_block(T + i0 + (size_t)i0 * NB, NB, sTb, w, w, w);
  }
  __syncthreads();
}

// --- the persistent executor ---------------------------------------------------------
// BATCH: the tasks of many matrices (FP64 tile kernels only); each task runs
// with its matrix's fields (s_b.lp).  Up to two CTAs per SM (at most 128
// registers per thread): while one runs a latency-bound panel column loop,
// the other's update keeps the FP64 pipe busy.
// OZG: t-groups of the split updates (8: FP64-level; 4: the reduced form).
// Thread 0: wait (bounded) until panel block `id` has finished its trailing
// update; false (error word set) when the wait ran out or the DAG failed.
__device__ bool wait_ts_flag(const DagParams& p, int id) {
  const uint64_t t0 = global_ns();
  while (*((volatile const int*)(p.tsflag + id)) == 0) {
    if (*((volatile const unsigned*)(p.ctl + kErr)) != 0u) return false;
    if ((long long)(global_ns() - t0) > p.timeout_ns) {
      atomicOr((int*)(p.ctl + kErr), kErrTimeout);
      return false;
    }
    __nanosleep(64);
  }
  return true;
}

// The phases of a factorization panel block with ts_split (see DagParams):
// called by every thread of the CTA at the points task_geqrt_blk /
// task_tsqrt_blk name.  Every wait is on a block that has already released
// this one (so it is running, past that release) and that waits only on
// blocks of smaller b or k itself: no cycle, and each wait is bounded.
// on == false: no phases (the block releases at its end, as without
// ts_split), and the trailing update keeps its usual column blocks.
struct PanelPhases {
  const DagParams* p;
  int i, k, b;
  bool on;
  __device__ int first_cols(int cb, int w) const { return on ? w : cb; }
  __device__ void publish() const {   // this CTA's writes, then thread 0 releases
    fence_acq_rel_gpu();
    __syncthreads();
  }
  __device__ void after_panel() const {   // R's diagonal block is final: the tile below's block b
    if (!on) return;
    publish();
    if (threadIdx.x == 0 && k + 1 < p->MT) release(*p, panel_id(*p, i, k + 1, b));
  }
  __device__ void before_trailing() const {
    if (!on) return;
    if (threadIdx.x == 0) {
      bool ok = true;
      if (b > 0) ok = wait_ts_flag(*p, panel_id(*p, i, k, b - 1));   // the same columns, earlier block
      if (ok && k > i) ok = wait_ts_flag(*p, panel_id(*p, i, k - 1, b));   // R's rows, tile above
      fence_acq_rel_gpu();   // acquire: their writes are visible
    }
    __syncthreads();
  }
  __device__ void after_first() const {   // the next block's columns are updated
    if (!on) return;
    publish();
    if (threadIdx.x == 0 && b + 1 < p->nblk) release(*p, panel_id(*p, i, k, b + 1));
  }
  __device__ void after_trailing() const {
    if (!on) return;
    publish();
    if (threadIdx.x == 0) atomicExch(p->tsflag + panel_id(*p, i, k, b), 1);
  }
};

// P32: the panel blocks compute in FP32 (HQR_PREC_FP32).
template <bool OZ, bool BATCH = false, int OZG = 8, bool P32 = false>
__global__ void __launch_bounds__(kThreads, BATCH ? 2 : 1) dag_exec_kernel(DagParams p) {
  using PanelT = typename std::conditional<P32, float, double>::type;
  extern __shared__ __align__(1024) double smem[];
  __shared__ int s_id;
  __shared__ uint32_t s_tmem;
  __shared__ BatchLocal<BATCH> s_b;
  unsigned long long local_cnt[kNumStats] = {0, 0, 0, 0, 0, 0, 0};
  unsigned long long local_cyc[kNumStats] = {0, 0, 0, 0, 0, 0, 0};
  if (OZ) {
    // the whole TMEM of this SM (one CTA per SM): 8 t-group accumulators x 64 columns
    if ((threadIdx.x >> 5) == 0) oz::tmem_alloc(&s_tmem, 512);
    oz::tc_fence_before();
    __syncthreads();
    oz::tc_fence_after();
  }
  init_local(s_b);
  int next = -1;   // thread 0: a continuation kept from the last release
  bool cont_ok = false;   // thread 0: no error and no high-priority task waiting (read before the releases)
  for (;;) {
    const long long cp = clock64();
    if (threadIdx.x == 0) {
      // A kept continuation runs next unless a high-priority task is waiting:
      // then it goes to the queue like any other ready task.
      if (next >= 0 && cont_ok) {
        fence_acq_rel_gpu();   // acquire: the other producers' tile writes are visible
        s_id = next;
      } else {
        if (next >= 0) push_queue(p, next, false);   // a kept task is never high-priority
        s_id = pop_task(p);
      }
      next = -1;
    }
    __syncthreads();
    const int gid = s_id;
    __syncthreads();
    if (gid < 0) break;
    load_local(p, s_b, gid);
    const DagParams& q = local_params(p, s_b);
    const int id = gid - q.id_base;
    const int NB = q.sh.NB;
    const size_t tsz = (size_t)NB * NB;
    const TaskDesc t = decode(q, id);
    const long long c0 = clock64();
    if (threadIdx.x == 0) local_cyc[kStatSched] += (unsigned long long)(c0 - cp);
    // Each heavy task body has one call site (the split engine, the panel
    // preparation and the TS/TT panel block are large when inlined): the
    // cases only pick their operands.
    const uint8_t* oz_slices = nullptr;   // an update on the tensor cores
    const int* oz_exps = nullptr;
    double *oz_top = nullptr, *oz_bot = nullptr;
    long long oz_col0 = 0;   // column of C where the update's first chunk starts
    const double *prep_v = nullptr, *prep_tau = nullptr;   // a split panel preparation
    double* prep_g = nullptr;
    uint8_t* prep_slices = nullptr;
    int* prep_exps = nullptr;
    int prep_kind = kVDense;
    double *ts_a1 = nullptr, *ts_a2 = nullptr, *ts_t = nullptr, *ts_tau = nullptr;   // a TS/TT panel block
    bool ts_upper = false;
    switch (t.type) {
      case kGEQRT: {   // the diagonal tile or a domain's top tile
        const size_t o = tile_off(t.k, t.i, q.MT, NB);
        task_geqrt_blk<PanelT>(q.A + o, q.T + o, q.TAU + tau_off(t.k, t.i, q.MT, NB), q.sh, smem, q.sp, t.c,
                               PanelPhases{&q, t.i, t.k, t.c, q.ts_split != 0 && t.i >= q.ts_split_from});
        break;
      }
      case kTSQRT: {   // R of the domain's top tile over tile (k, i)
        const int top = dom_top(q, t.i, dom_of(q, t.i, t.k));
        const size_t o2 = tile_off(t.k, t.i, q.MT, NB);
        ts_a1 = q.A + tile_off(top, t.i, q.MT, NB);
        ts_a2 = q.A + o2;
        ts_t = q.T + o2;
        ts_tau = q.TAU + tau_off(t.k, t.i, q.MT, NB);
        break;
      }
      case kTTQRT: {   // merge of domain top t.k's R into R(i, i): FP64 on the panel path
        const size_t slot = merge_slot(q, t.i, dom_of(q, t.i, t.k));
        ts_a1 = q.A + tile_off(t.i, t.i, q.MT, NB);
        ts_a2 = q.A + tile_off(t.k, t.i, q.MT, NB);
        ts_t = q.T2 + slot * tsz;
        ts_tau = q.TAU2 + slot * NB;
        ts_upper = true;
        break;
      }
      case kTBUILD: {
        const size_t o = tile_off(t.k, t.i, q.MT, NB);
        task_tbuild(q.A + o, q.TAU + tau_off(t.k, t.i, q.MT, NB), q.T + o, t.k == t.i, q.sh, smem, q.sp);
        break;
      }
      case kOZPREP: {
        const size_t o = tile_off(t.k, t.i, q.MT, NB);
        const size_t slot = panel_slot(q.MT, t.i, t.k);
        prep_v = q.A + o;
        prep_tau = q.TAU + tau_off(t.k, t.i, q.MT, NB);
        prep_g = q.T + o;
        prep_kind = is_top(q, t.i, t.k) ? kVUnitLower : kVDense;
        prep_slices = q.slices + slot * oz::panel_slice_bytes();
        prep_exps = q.sexp + slot * oz::kSlots * NB;
        break;
      }
      case kTTPREP: {
        const size_t slot = merge_slot(q, t.i, dom_of(q, t.i, t.k));
        prep_v = q.A + tile_off(t.k, t.i, q.MT, NB);
        prep_tau = q.TAU2 + slot * NB;
        prep_g = q.T2 + slot * tsz;
        prep_kind = kVUpper;
        prep_slices = q.slices2 + slot * oz::panel_slice_bytes();
        prep_exps = q.sexp2 + slot * oz::kSlots * NB;
        break;
      }
      case kLARFB: {   // tile row k = the diagonal or a domain top
        const size_t ov = tile_off(t.k, t.i, q.MT, NB), oc = tile_off(t.k, t.j, q.MT, NB);
        if (OZ) {
          const size_t slot = panel_slot(q.MT, t.i, t.k);
          oz_slices = q.slices + slot * oz::panel_slice_bytes();
          oz_exps = q.sexp + slot * oz::kSlots * NB;
          oz_bot = q.C + oc + (size_t)t.c * q.oz_cpt * oz::kN * NB;
          oz_col0 = (long long)t.j * NB + (long long)t.c * q.oz_cpt * oz::kN;
        } else if (q.c_cols <= 0 || (long long)t.j * NB + (long long)t.c * q.sh.CB < q.c_cols) {
          task_larfb(q.A + ov, q.T + ov, q.C + oc, t.c * q.sh.CB, q.sh.CB, q.sh, smem, q.sp,
                     applies_h(q.mode));
        }
        break;
      }
      case kSSRFB:     // A1 = the domain top's tile row
      case kTTMQR: {   // the merge's reflectors on [row i; the domain top's row] of column j
        const bool tt = t.type == kTTMQR;
        const int top = tt ? t.i : dom_top(q, t.i, dom_of(q, t.i, t.k));
        const size_t ov = tile_off(t.k, t.i, q.MT, NB);
        const size_t o1 = tile_off(top, t.j, q.MT, NB), o2 = tile_off(t.k, t.j, q.MT, NB);
        const size_t slot = tt ? merge_slot(q, t.i, dom_of(q, t.i, t.k)) : panel_slot(q.MT, t.i, t.k);
        if (OZ) {
          const size_t cofs = (size_t)t.c * q.oz_cpt * oz::kN * NB;
          oz_slices = (tt ? q.slices2 : q.slices) + slot * oz::panel_slice_bytes();
          oz_exps = (tt ? q.sexp2 : q.sexp) + slot * oz::kSlots * NB;
          oz_top = q.C + o1 + cofs;
          oz_bot = q.C + o2 + cofs;
          oz_col0 = (long long)t.j * NB + (long long)t.c * q.oz_cpt * oz::kN;
        } else if (q.c_cols <= 0 || (long long)t.j * NB + (long long)t.c * q.sh.CB < q.c_cols) {
          task_ssrfb(q.C + o1, q.C + o2, q.A + ov, tt ? q.T2 + slot * tsz : q.T + ov, t.c * q.sh.CB,
                     q.sh.CB, q.sh, smem, q.sp, applies_h(q.mode), tt);
        }
        break;
      }
      default:
        if (threadIdx.x == 0) atomicOr((int*)(q.ctl + kErr), kErrBadTask);
    }
    if (ts_a1)
      task_tsqrt_blk<PanelT>(ts_a1, ts_a2, ts_t, ts_tau, q.sh, smem, q.sp, t.c, ts_upper,
                             PanelPhases{&q, t.i, t.k, t.c, q.ts_split != 0 && t.i >= q.ts_split_from && !ts_upper});
    // Q generation and Q C apply H (M = T), the other modes H^T (M = T^T)
    if (OZ && prep_v)
      task_ozprep(prep_v, prep_tau, prep_g, prep_kind, prep_slices, prep_exps, reinterpret_cast<uint8_t*>(smem),
                  s_tmem, q.ctl + kErr, !applies_h(q.mode));
    if (OZ && oz_bot) {
      for (int cc = 0; cc < q.oz_cpt; cc++) {
        if (q.c_cols > 0 && oz_col0 + (long long)cc * oz::kN >= q.c_cols) break;
        const size_t co = (size_t)cc * oz::kN * NB;
        oz::Ctx c;
        oz::ctx_init(c, reinterpret_cast<uint8_t*>(smem), s_tmem, q.ctl + kErr);
        if (!task_ozapply<OZG>(c, oz_slices, oz_exps, oz_top ? oz_top + co : nullptr, oz_bot + co)) break;
      }
    }
    fence_acq_rel_gpu();   // release: this task's writes before its dependents' counters
    __syncthreads();
    if (threadIdx.x == 0) {
      local_cnt[stat_slot(t.type)]++;
      const long long c1 = clock64();
      local_cyc[stat_slot(t.type)] += (unsigned long long)(c1 - c0);
      // the control words are read before the releases so that their round
      // trips overlap the releases' atomics
      volatile unsigned* ctl = q.ctl;
      const unsigned err_now = ctl[kErr], hi_head = ctl[kHiHead], hi_tail = ctl[kHiTail];
      const bool pushed_hi = release_dependents(q, t, &next);
      cont_ok = err_now == 0u && hi_head >= hi_tail && !pushed_hi;
      atomicAdd(q.ctl + kDone, 1u);   // termination count only: no ordering needed
      local_cnt[kStatSched]++;
      local_cyc[kStatSched] += (unsigned long long)(clock64() - c1);
    }
  }
  if (threadIdx.x == 0 && p.stats) {
    for (int ty = 0; ty < kNumStats; ty++) {
      if (local_cnt[ty]) {
        atomicAdd(p.stats + 2 * ty, local_cnt[ty]);
        atomicAdd(p.stats + 2 * ty + 1, local_cyc[ty]);
      }
    }
  }
  if (OZ) {
    oz::tc_fence_before();
    __syncthreads();
    oz::tc_fence_after();
    if ((threadIdx.x >> 5) == 0) oz::tmem_dealloc(s_tmem, 512);
  }
}

}  // namespace hqr
