/*
 * tile_kernel.h -- the reference's own tile kernels (Hybrid3 tile_kernel.h:28-230,
 * bodies tile_kernel.c:19-716), same prototypes, executed on the GPU.
 *
 * Pointer arguments may be host or device memory: device (or managed)
 * pointers are used in place; host pointers are staged through device memory
 * for the call.  `work` is accepted for signature compatibility and is not
 * needed (tile_init still returns a 3*row*col double buffer, tile_kernel.c:19-25).
 *
 * These kernels keep the reference's own conventions, which differ from the
 * factorization path (Hybrid_tile_QR, which follows LAPACK dlarfg):
 *   - reflector: beta = +||x||, y = [alpha - beta; x], v = y / y(0),
 *     tau = 2 y(0)^2 / ||y||^2; no guard for x = 0 (alpha > 0 divides by 0);
 *   - T is LOWER triangular, the transpose of LAPACK's forward T:
 *     T(i,i) = tau_i, T(i,0:i) = -tau_i (T(0:i,0:i)^T (Y^T y_i)(0:i));
 *   - tile_sub_dgeqr2 with row == col leaves TAU[col-1] unwritten and sets
 *     Y(col-1,col-1) = 0;
 *   - tile_dgeqrt builds only the diagonal T blocks;
 *   - tile_dlarft with 2 <= block < col couples all blocks but the last;
 *     block >= col leaves T untouched;
 *   - tile_sub_dlarfb uses the stored diagonal of Y (a unit diagonal must be
 *     stored explicitly) and applies I - Y T Y^T (the transpose of the Q the
 *     reflectors form);
 *   - tile_sub_dssrfb with over_row > Y_col zeroes rows Y_col.. of A1.
 */
#ifndef HYBRID3_GB300_TILE_KERNEL_H_
#define HYBRID3_GB300_TILE_KERNEL_H_
#include <stdio.h>
#include <stdlib.h>
#include <math.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* tile_kernel.c:19: calloc of 3*tile_row*tile_col doubles ('d' only). */
void *tile_init(char type, int tile_row, int tile_col);

/* tile_kernel.c:28: blocked QR of one tile with the repo's conventions. */
void tile_dgeqrt(const int row, const int col, const int block, double *A, const int lda,
                 double *TAU, double *Y, double *T, const int ldt, double *work);
/* tile_kernel.c:60: QR of [A1 (upper); A2]. */
void tile_dtsqrt(const int row, const int col, const int block, double *A1, const int lda1,
                 double *A2, const int lda2, double *TAU, double *T, const int ldt, double *work);
/* tile_kernel.c:106: A <- (I - Y T Y^T) A with the dgeqrt (Y, T). */
void tile_dlarfb(const int row, const int col, double *A, const int lda, const double *Y,
                 const double *T, const int ldt, double *work);
/* tile_kernel.c:121: [A1; A2] <- (I - [I;Y] T [I;Y]^T) [A1; A2] with the tsqrt (Y, T). */
void tile_dssrfb(const int row, const int col, double *A1, double *A2, const int lda,
                 const double *Y, const double *T, const int ldt, double *work);
/* tile_kernel.c:138: unblocked QR (repo convention). */
void tile_sub_dgeqr2(const int row, const int col, double *A, const int lda, double *TAU,
                     double *Y, double *work);
/* tile_kernel.c:220: lower T from Y and TAU. */
void tile_sub_dlarft(const int row, const int col, const double *Y, const int lda,
                     const double *TAU, double *T, const int ldt, double *work);
/* tile_kernel.c:264: A(row x A_col) <- (I - Y T Y^T) A. */
void tile_sub_dlarfb(const int row, const int Y_col, const int A_col, const double *Y,
                     const int ldy, const double *T, const int ldt, double *A, const int lda,
                     double *work);
/* tile_kernel.c:313: [A1; A2] <- (I - [I;Y] T [I;Y]^T) [A1; A2]. */
void tile_sub_dssrfb(const int over_row, const int under_row, const int Y_col, const int A_col,
                     const double *Y, const int ldy, const double *T, const int ldt, double *A1,
                     const int lda1, double *A2, const int lda2, double *work);
/* tile_kernel.c:368: lower T, optionally in blocks. */
void tile_dlarft(const int row, const int col, const int block, const double *Y, const int lda,
                 const double *TAU, double *T, const int ldt, double *work);
/* tile_kernel.c:439: first half of tile_dssrfb (A1 update, W kept in upper_mat). */
void tile_dssrfb_head(const int row, const int col, double *A1, double *A2, const int lda,
                      const double *Y, const double *T, const int ldt, double *upper_mat);
/* tile_kernel.c:478: second half (A2 -= Y W). */
void tile_dssrfb_tail(const int row, const int col, double *A2, const int lda, const double *Y,
                      double *upper_mat);
/* tile_kernel.c:501: tile_dlarfb with T read row-major (T^T of the column-major array). */
void tile_return_dlarfb(const int row, const int col, double *A, const int lda, const double *Y,
                        const double *T, const int ldt, double *work);
/* tile_kernel.c:603: tile_dssrfb with T read row-major. */
void tile_return_dssrfb(const int row, const int col, double *A1, double *A2, const int lda,
                        const double *Y, const double *T, const int ldt, double *work);
/* Declared at tile_kernel.h:216 of the reference but never defined there;
 * here it is tile_sub_dlarft with T stored transposed (upper, as read by the
 * tile_return_* kernels). */
void tile_return_dlarft(const int row, const int col, const double *Y, const int lda,
                        const double *TAU, double *T, const int ldt, double *work);
/* tile_kernel.c:654: unblocked QR of [A1 (upper); A2] (repo convention). */
void tile_sub_dtsqr2(const int row, const int col, double *A1, const int lda1, double *A2,
                     const int lda2, double *TAU, double *work);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif
