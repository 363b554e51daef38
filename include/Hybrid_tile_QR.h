/*
 * Hybrid_tile_QR.h -- drop-in C entry points of the tiled Householder QR
 * (Hybrid3's Hybrid_tile_QR.h:19-77), executed on one GB300 GPU.
 *
 * All arrays are HOST arrays in the tile layout of mat_prod.h, allocated and
 * (for Q) zero-initialised by the caller, exactly as with the reference; each
 * call copies its operands to the GPU, runs the tile DAG there and copies the
 * results back.  Only one rank is supported: Proc_num must be 1 and my_rank 0
 * (the reference's MPI distribution is collapsed onto one device).
 *
 * Errors are printed to stderr and end the process, like the reference's
 * MPI_Abort, unless hqr_set_error_mode(HQR_ERRORS_RETURN) was called; then the
 * call returns and hqr_last_error() reports the status.
 */
#ifndef HYBRID3_GB300_HYBRID_TILE_QR_H_
#define HYBRID3_GB300_HYBRID_TILE_QR_H_
#include <stdio.h>
#include <stdlib.h>
#include "mat_prod.h"
#include "tile_kernel.h"

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* Declared but never defined by the reference (Hybrid_tile_QR.h:19-24); here
 * it is Hybrid_tile_QR with ib = NB, the reference driver's default
 * (main.c:85-88). */
void Hybrid_dgeqrf(mat_stat_t *status, double *A, double *TAU, int my_rank, int Proc_num);

/* Hybrid_tile_QR.c:307: in-place tiled QR.  On return A holds R on and above
 * the diagonal and the Householder vectors V below it (unit diagonal
 * implicit); TAU holds NB scalars per panel tile at mat_getVecPos(status,i,j). */
void Hybrid_tile_QR(mat_stat_t *status, double *A, double *TAU, int my_rank, int Proc_num, int ib);

/* Hybrid_make_Q.c:56: Q (zeroed by the caller) receives Q^T = H_last^T..H_1^T I;
 * the reflectors are zeroed in RY, which becomes R. */
void Hybrid_make_Q(mat_stat_t *status, double *Q, double *RY, double *TAU, int my_rank,
                   int Proc_num, int ib);

/* Hybrid_make_I.c:20: identity in tile layout (the whole array is written). */
void Hybrid_make_I(mat_stat_t *status, double *Id, int my_rank, int Proc_num);

/* Declared but never defined by the reference (Hybrid_tile_QR.h:47-53); here
 * it zeroes the reflectors V below the diagonal of the factored RY, leaving R,
 * as Hybrid_make_Q does (Hybrid_make_Q.c:148-150,179-182). */
void Hybrid_remv_Y(mat_stat_t *status, double *RY, int my_rank, int Proc_num);

/* Hybrid_dgemm.c:16: tile-wise C = A^T B of two square tiled matrices. */
void Hybrid_dgemm(mat_stat_t *status, double *A, double *B, double *C, int my_rank, int Proc_num);

/* Hybrid_dorgqr.c:22: Q <- Q^T of the factorization (Q is overwritten; RY and
 * TAU are left unchanged). */
void Hybrid_dorgqr(mat_stat_t *status, double *Q, double *RY, double *TAU, int my_rank,
                   int Proc_num);

/* Hybrid_dormqr.c:20: C <- Q^T C, C in the same tile grid as RY. */
void Hybrid_dormqr(mat_stat_t *status, double *RY, double *TAU, double *C, int my_rank,
                   int Proc_num);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif
