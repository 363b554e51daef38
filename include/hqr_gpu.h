/*
 * hqr_gpu.h -- extended C ABI of the GB300 tiled Householder QR.
 *
 * The drop-in entry points (Hybrid_tile_QR.h) take host arrays and end the
 * process on error, as the reference does.  This interface is what they are
 * built on: device pointers, CUDA streams (passed as void*), integer status
 * codes, persisted T factors and a choice of arithmetic for the trailing
 * updates.  All matrices use the tile layout of mat_prod.h (tile (i,j) of an
 * MT x NT grid of NB x NB column-major tiles at (i + j*MT)*NB*NB; TAU block of
 * tile (i,j) at (i + j*MT)*NB).
 */
#ifndef HYBRID3_GB300_HQR_GPU_H_
#define HYBRID3_GB300_HQR_GPU_H_
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* Status codes. */
#define HQR_OK 0
#define HQR_ERR_INVALID (-1)     /* bad argument (shape, pointer, rank count) */
#define HQR_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define HQR_ERR_TIMEOUT (-3)     /* a bounded device wait ran out (scheduler) */
#define HQR_ERR_NOMEM (-4)       /* device allocation failed */
#define HQR_ERR_UNSUPPORTED (-5) /* shape outside what the kernels support */
#define HQR_ERR_DEVICE (-6)      /* a device-side consistency check failed */

/* Arithmetic of the trailing updates (and, for HQR_PREC_FP32, of the panels). */
#define HQR_PREC_FP64 0    /* FP64 on CUDA cores */
#define HQR_PREC_OZAKI 1   /* split-precision slices on the tensor cores, FP64 recombination;
                              NB = 128 only (HQR_ERR_UNSUPPORTED otherwise) */
#define HQR_PREC_OZAKI_FAST 2 /* the same updates with only the slice products of weight <= 3
                              (10 of 36): each product to about 2^-30 of its operands' row and
                              column maxima, an FP32-class factorization (FP64 panels, NB = 128
                              only).  For least squares with FP64 iterative refinement
                              (hqr_lstsq, refine_steps >= 2) on well-conditioned problems: the
                              refinement ends near kappa^2 * 5e-9 * ||r|| / (||A|| ||x||);
                              hqr_lstsq_aug refines to the FP64 solution instead */
#define HQR_PREC_FP32 3       /* an FP32-class factorization: the panel blocks (GEQRT / TSQRT
                              and their in-tile updates) compute in FP32 on values kept in
                              FP64 arrays, the updates are those of HQR_PREC_OZAKI_FAST; the
                              reference's FP32 factorization for least squares refined in
                              FP64 (hqr_lstsq_aug).  NB = 128 only */

/* Error behaviour of the drop-in (Hybrid_*, tile_*) entry points. */
#define HQR_ERRORS_ABORT 0   /* print to stderr and exit(1) (the reference's MPI_Abort) */
#define HQR_ERRORS_RETURN 1  /* print to stderr and return; see hqr_last_error() */

typedef struct hqr_plan hqr_plan_t;

/* Per-task-type execution counters of the last DAG run (device clock cycles
 * summed over CTAs).  Index: 0 GEQRT, 1 TSQRT, 2 LARFB, 3 SSRFB, 4 T-build,
 * 5 split-precision panel preparation (full T + operand slices), 6 the
 * scheduler itself (thread 0 of each CTA popping tasks and releasing their
 * dependents; count = tasks).  GEQRT and TSQRT are counted per inner block
 * of w = min(IB, 32) columns (w = 16 with HQR_PREC_OZAKI): each inner block is
 * its own task. */
typedef struct {
    unsigned long long count[7];
    unsigned long long cycles[7];
} hqr_stats_t;

const char *hqr_status_string(int status);
void hqr_set_error_mode(int mode);
/* Arithmetic of the trailing updates used by the drop-in entry points
 * (default: HQR_PREC_FP64, or HQR_PREC_OZAKI when the environment variable
 * HQR_PRECISION is "ozaki" or "split" at first use, HQR_PREC_OZAKI_FAST when
 * it is "fast"). */
void hqr_set_default_precision(int precision);
int hqr_get_default_precision(void);
int hqr_last_error(void);
/* Text of the last failed CUDA runtime call ("" if none). */
const char *hqr_last_cuda_error(void);
/* Device-side wait limit of the scheduler, in milliseconds (default 20000). */
void hqr_set_timeout_ms(long long ms);

/* A plan owns the device workspace for one (M, N, NB, IB, precision) shape:
 * T factors of every panel tile (M*N doubles), the DAG's dependency counters
 * and ready queues.  M and N must be multiples of NB; NB a multiple of 16 up
 * to 512; IB a divisor of NB (inner blocks of min(IB, 32) columns are used). */
int hqr_plan_create(hqr_plan_t **plan, long M, long N, int NB, int IB, int precision);
int hqr_plan_destroy(hqr_plan_t *plan);
/* No counterpart in the reference (its TS reduction is the flat tree).  Domain
 * tree for the factorizations on this plan: at step i the tile rows i.. are
 * cut into domains of domain_tiles tiles; each domain runs the flat TS chain
 * on its own top tile (GEQRT + TSQRT), then the domain tops' R are merged into
 * R(i, i) one after the other by triangle-on-triangle QRs (CORE_dttqrt /
 * CORE_dttmqr).  The TS chain down a panel shrinks from MT - i tiles to
 * domain_tiles + the number of domains, for tall-skinny matrices.  0 (the
 * default) or domain_tiles >= MT: the flat tree of the reference.  With a tree,
 * R is the same (up to the signs of its rows) but the reflectors differ: the
 * merges' T factors and TAU live in the plan, so hqr_ormqr_t and hqr_make_q
 * need use_plan_t = 1 (HQR_ERR_UNSUPPORTED otherwise) and Q is built by the
 * forward application.  Allocates the merges' storage. */
int hqr_plan_set_tree(hqr_plan_t *plan, int domain_tiles);
/* Device T factors: one NB x NB tile per panel tile, same tile layout as A.
 * FP64: the last factorization's w x w diagonal blocks of T (upper
 * triangular).  Split precision: the whole NB x NB operand of the last call
 * that prepared operands -- T^T after hqr_geqrf / hqr_ormqr_t, T after Q
 * generation or hqr_ormqr_n. */
double *hqr_plan_t_factors(hqr_plan_t *plan);

/* In-place factorization of dA (device), TAU to dTAU (MT*NT*NB doubles).
 * hqr_geqrf waits for completion and reports device-side errors;
 * hqr_geqrf_async only enqueues (check with hqr_plan_status). */
int hqr_geqrf(hqr_plan_t *plan, double *dA, double *dTAU, void *stream);
int hqr_geqrf_async(hqr_plan_t *plan, double *dA, double *dTAU, void *stream);
/* No counterpart in the reference.  The factorization of hqr_geqrf for callers
 * that may not allocate device memory (a process whose device memory is owned
 * entirely by its own pool allocator, a latency path that cannot take the
 * device-wide synchronisation an allocation may cause): it calls no
 * cudaMalloc/cudaFree and uses a fixed 64 MiB scratch array that the library
 * reserves on each GPU that loads it, for the T factors (M*N doubles) and the
 * scheduler tables -- shapes that do not fit (about n > 2800 square) return
 * HQR_ERR_UNSUPPORTED.  All calls share that array: calls that overlap on the
 * GPU race, so serialise them.  The first call on a device looks the array's
 * address up; make that call before any stream capture.  Each call waits for
 * `stream` to finish (it synchronises it) and returns the scheduler's status. */
int hqr_geqrf_noalloc(long M, long N, int NB, int IB, double *dA, double *dTAU, void *stream);
/* Synchronise `stream`, then read and clear the scheduler's error word. */
int hqr_plan_status(hqr_plan_t *plan, void *stream);
int hqr_plan_stats(hqr_plan_t *plan, hqr_stats_t *out, void *stream);

/* Hybrid_make_Q semantics on device arrays: dQ (M x N) <- Q^T I; the
 * reflectors of dRY are zeroed (dRY becomes R).  use_plan_t = 1: dRY and dTAU
 * are the output of the last hqr_geqrf on this plan, and its T factors (FP64)
 * or prepared operands (split precisions), kept in the plan, are used as they
 * are -- no panel tasks run.  If a call since then rebuilt them from other
 * reflectors (use_plan_t = 0 here or in hqr_ormqr_t, or a drop-in Hybrid_*
 * call), they are rebuilt from dRY and dTAU instead.  use_plan_t = 0: always
 * rebuilt from dRY and dTAU (any reflectors in this plan's shape), replacing
 * the plan's.  Square Q generation applies H itself, not H^T: with a split
 * precision its prepared operands ([T V^T | T], where the factorization and
 * Q^T C use [T^T V^T | T^T]) are made by its first call after a
 * factorization and kept apart, so later calls reuse them. */
int hqr_make_q(hqr_plan_t *plan, double *dQ, double *dRY, const double *dTAU, int use_plan_t,
               void *stream);
int hqr_make_q_async(hqr_plan_t *plan, double *dQ, double *dRY, const double *dTAU,
                     int use_plan_t, void *stream);
/* Hybrid_dormqr semantics: dC <- Q^T dC, dC an MT x CT tile grid (CT tile
 * columns of NB, e.g. CT = 1 for up to NB right-hand sides padded to NB).
 * use_plan_t as for hqr_make_q.  hqr_ormqr_t waits for completion;
 * hqr_ormqr_t_async only enqueues (check with hqr_plan_status). */
int hqr_ormqr_t(hqr_plan_t *plan, const double *dRY, const double *dTAU, double *dC, int CT,
                int use_plan_t, void *stream);
int hqr_ormqr_t_async(hqr_plan_t *plan, const double *dRY, const double *dTAU, double *dC, int CT,
                      int use_plan_t, void *stream);
/* No counterpart in the reference (its dormqr applies Q^T only).  dC <- Q dC
 * (LAPACK dormqr 'L','N'): the reflectors applied as H, in backward order,
 * to every tile column of dC (MT x CT tiles).  use_plan_t as for hqr_make_q;
 * split precisions keep the prepared operands of H apart from those of H^T,
 * so Q dC and Q^T dC both reuse theirs after one preparation.  Flat tree
 * only (HQR_ERR_UNSUPPORTED with a domain tree).  The _async form only
 * enqueues (check with hqr_plan_status). */
int hqr_ormqr_n(hqr_plan_t *plan, const double *dRY, const double *dTAU, double *dC, int CT,
                int use_plan_t, void *stream);
int hqr_ormqr_n_async(hqr_plan_t *plan, const double *dRY, const double *dTAU, double *dC, int CT,
                      int use_plan_t, void *stream);

/* No counterpart in the reference (its driver stops at Q and R).  Least
 * squares min ||A x - b||_2 for a full-rank dA (M >= N, tile layout of this
 * plan's shape, device, left unmodified) and nrhs right-hand sides dB
 * (column-major M x nrhs, ld ldb >= M, device): a copy of A is factored on
 * this plan (its precision), c = Q^T b runs on the device DAG (dormqr), R x =
 * c(1:N) is solved by blocked back substitution, then refine_steps steps of
 * FP64 iterative refinement: r = b - A x with the original A in FP64, x +=
 * R^-1 (Q^T r)(1:N).  dX: column-major N x nrhs (ld ldx >= N, device).
 * resid (host, nrhs doubles, may be NULL) receives ||b - A x||_2 of the
 * returned x per right-hand side.  Its workspace (the copy of A, TAU, the
 * packed right-hand sides) is allocated on the plan by the first call, kept
 * for later calls (grown if they need more) and freed with the plan.
 * Synchronous: returns the scheduler's status. */
int hqr_lstsq(hqr_plan_t *plan, const double *dA, const double *dB, int ldb, int nrhs, double *dX,
              int ldx, int refine_steps, double *resid, void *stream);
/* No counterpart in the reference.  hqr_lstsq's arguments and result, refined
 * on the augmented system [I A; A^T 0][r; x] = [b; 0] (Bjorck): x0 and r0 =
 * b - A x0 as above, then each of refine_steps steps forms f = b - r - A x
 * and g = -A^T r in FP64 and solves for the correction with the factorization:
 * h = R^-T g, d = Q^T f (hqr_ormqr_t), x += R^-1 (d(1:N) - h), r += Q [h;
 * d(N+1:M)] (hqr_ormqr_n).  The limit of x is the FP64 least-squares
 * solution's accuracy (about kappa(A) u in FP64, plus kappa^2 u ||r|| /
 * (||A|| ||x||)) whatever the factorization's precision, as long as the
 * factorization's error times kappa(A) stays below about 0.1; hqr_lstsq's
 * refinement stalls at the factorization's error times kappa(A) ||r|| /
 * (||A|| ||x||) instead.  HQR_ERR_UNSUPPORTED with a domain tree.  Workspace
 * as for hqr_lstsq (plus two tile grids of the right-hand sides and the
 * residual r); synchronous. */
int hqr_lstsq_aug(hqr_plan_t *plan, const double *dA, const double *dB, int ldb, int nrhs, double *dX,
                  int ldx, int refine_steps, double *resid, void *stream);

/* No counterpart in the reference (it factors one matrix per run).  A batch
 * of independent FP64 tile QRs of uneven shapes, each run of the batch one
 * persistent launch of the DAG executor over every matrix's tasks (a
 * per-matrix task table: tile counts, tile order, arrays, first task id).
 * Matrix b is M[b] x N[b] in the NB[b] x NB[b] tile layout of hqr_geqrf (M, N
 * multiples of NB[b]; zero padding to such a shape leaves the leading block
 * of R and the reflectors unchanged), inner blocks min(IB[b], 32).  max_nrhs:
 * the largest nrhs that hqr_batch_ormqr_t will be given (its scheduler tables
 * are reserved here, so a call can be captured into a CUDA graph).
 * ctas_per_sm: executor CTAs per SM.  2 runs two on each SM (while one is in
 * a latency-bound panel column loop the other's update keeps the FP64 pipe
 * busy); every matrix's tile plan must then fit half an SM's shared memory
 * (the update tasks' column blocks narrow to fit; NB <= 128 with inner blocks
 * of 16, NB <= 64 with 32), else HQR_ERR_UNSUPPORTED.  1: one per SM, the
 * widest column blocks.  0: 2 when every matrix fits, else 1.  The batch
 * owns the T factors of every matrix. */
typedef struct hqr_batch hqr_batch_t;
int hqr_batch_create(hqr_batch_t **batch, int count, const long *M, const long *N, const int *NB,
                     const int *IB, int max_nrhs, int ctas_per_sm);
int hqr_batch_destroy(hqr_batch_t *batch);
/* Factor every matrix in place: dA[b], dTAU[b] (MT*NT*NB doubles) are device
 * pointers held in a host array.  The _async form only enqueues; the first
 * call with a new set of pointers uploads the task table and may not be
 * captured into a graph (HQR_ERR_UNSUPPORTED): later calls with the same
 * pointers enqueue kernels and memsets only. */
int hqr_batch_geqrf(hqr_batch_t *batch, double *const *dA, double *const *dTAU, void *stream);
int hqr_batch_geqrf_async(hqr_batch_t *batch, double *const *dA, double *const *dTAU, void *stream);
/* Hybrid_dormqr for every matrix: the first nrhs columns of dC[b] <- Q_b^T
 * dC[b] for the last factorization of the batch (its T factors).  dC[b] is an
 * MT x ceil(nrhs / NB[b]) tile grid of NB[b] tiles; its columns from nrhs on
 * may or may not be transformed.  nrhs <= max_nrhs. */
int hqr_batch_ormqr_t(hqr_batch_t *batch, double *const *dA, double *const *dTAU, double *const *dC,
                      int nrhs, void *stream);
int hqr_batch_ormqr_t_async(hqr_batch_t *batch, double *const *dA, double *const *dTAU,
                            double *const *dC, int nrhs, void *stream);
/* Executor CTAs per SM of the batch's launches (1 or 2). */
int hqr_batch_ctas_per_sm(hqr_batch_t *batch);
/* Synchronise `stream`, then read and clear the batch scheduler's error word. */
int hqr_batch_status(hqr_batch_t *batch, void *stream);
/* Task counts and SM cycles of the batch's last run (as hqr_plan_stats). */
int hqr_batch_stats(hqr_batch_t *batch, hqr_stats_t *out, void *stream);

/* Tile-wise C = A^T B of square tiled matrices (Hybrid_dgemm). */
int hqr_dgemm_tn(long N, int NB, const double *dA, const double *dB, double *dC, void *stream);
/* Identity in tile layout (Hybrid_make_I). */
int hqr_make_identity(long M, long N, int NB, double *dQ, void *stream);
/* Seeded i.i.d. uniform[-1,1) matrix in tile layout: element (r, c) is
 * 2u-1, u = top 53 bits of splitmix64(r + c*M + (seed+1)*0x9E3779B97F4A7C15). */
int hqr_fill_uniform(long M, long N, int NB, uint64_t seed, double *dA, void *stream);
/* ||X - Y - alpha*I||_F^2 over tiled arrays (Y may be NULL), result on the host. */
int hqr_frob2(long M, long N, int NB, const double *dX, const double *dY, double alpha,
              double *result, void *stream);
/* Tile layout <-> column-major (ld = M). */
int hqr_tiles_to_colmajor(long M, long N, int NB, const double *dT, double *dCM, void *stream);
int hqr_colmajor_to_tiles(long M, long N, int NB, const double *dCM, double *dT, void *stream);
/* Any M x N column-major matrix (leading dimension ld >= M) <-> the tile
 * layout padded to whole tiles: dT holds ceil(M/NB) x ceil(N/NB) tiles of
 * NB x NB, the rows and columns beyond M, N zero (to tiles) or ignored (from
 * tiles).  Zero padding leaves a QR's R (and Q's leading M x N block) that of
 * the unpadded matrix: the padded rows and columns add reflectors with tau 0.
 * The reference has a one-way printing version (mat_dprint, mat_prod.c:260). */
int hqr_colmajor_to_tiles_padded(long M, long N, long ld, int NB, const double *dCM, double *dT,
                                 void *stream);
int hqr_tiles_to_colmajor_padded(long M, long N, long ld, int NB, const double *dT, double *dCM,
                                 void *stream);
/* The split-precision product engine on its own (diagnostics / tests):
 * dC = dX dY for dX NB x NB and dY NB x 64, column-major device arrays,
 * NB = 128; same slicing, tensor-core products and recombination as
 * the HQR_PREC_OZAKI updates.  Synchronous. */
int hqr_ozaki_product(int NB, const double *dX, const double *dY, double *dC, void *stream);
/* No counterpart in the reference (its driver mallocs its arrays).  Page-locked
 * host memory (cudaHostAlloc) for the arrays given to the drop-in calls: their
 * host<->device copies then run at the link's full rate, on every call (they
 * are made by SM loads and stores through the arrays' device mapping).
 * Pageable memory works as well (cudaMemcpyAsync); so does memory the caller
 * locked by other means.  Free with hqr_host_free. */
int hqr_host_alloc(void **ptr, size_t bytes);
int hqr_host_free(void *ptr);
/* No counterpart in the reference: where the time of the last drop-in call
 * (Hybrid_tile_QR, Hybrid_make_Q, Hybrid_dorgqr, Hybrid_dormqr) went, in
 * milliseconds, from CUDA events on its stream: out[0] host-to-device copies,
 * out[1] the tile DAG, out[2] the stream idle while the host read the
 * scheduler's status, out[3] device-to-host copies, out[4] the device total,
 * out[5] the call's host wall time. */
int hqr_dropin_phase_ms(double *out);
/* Measured FP64 FMA issue rate of this GPU in TFLOP/s (a ~10 ms probe of
 * independent FMA chains): the roofline denominator of the FP64 kernels. */
double hqr_fp64_peak_tflops(void *stream);
/* The same for the FP64 tensor cores: mma.sync f64 (DMMA) on independent
 * accumulators, shape 0 = m8n8k4, 1 = m16n8k16; -1 on a bad shape or error. */
double hqr_fp64_mma_peak_tflops(int shape, void *stream);
/* Zero the reflectors below the diagonal (Hybrid_remv_Y). */
int hqr_zero_reflectors(long M, long N, int NB, double *dA, void *stream);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif
