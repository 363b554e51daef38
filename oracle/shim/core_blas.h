/* The four PLASMA CORE tile kernels the reference calls, restated through
 * their LAPACK (3.4+) equivalents, which compute the same factorization and
 * store T in the same layout (IB x IB upper blocks, one per IB columns, rows
 * 0..IB-1 of an LDT-leading array):
 *   CORE_dgeqrt -> dgeqrt      (TAU(j) is the diagonal of its T block)
 *   CORE_dtsqrt -> dtpqrt, l=0 (A1 upper triangular, A2 dense)
 *   CORE_dormqr -> dgemqrt     (left, transpose)
 *   CORE_dtsmqr -> dtpmqrt, l=0 (left, transpose)
 * Rounding may differ from PLASMA's own kernels at the last-bit level.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef HQR_SHIM_CORE_BLAS_H
#define HQR_SHIM_CORE_BLAS_H
#include "plasma.h"
#include "lapacke.h"

static inline void hqr_shim_tau_from_t(int n, int ib, const double *T, int ldt, double *tau)
{
    for (int j = 0; j < n; j++) tau[j] = T[(j % ib) + (long)j * ldt];
}
static inline int CORE_dgeqrt(int M, int N, int IB, double *A, int LDA, double *T, int LDT,
                              double *TAU, double *WORK)
{
    int k = M < N ? M : N;
    int ib = IB < k ? IB : k;
    int info = scipy_LAPACKE_dgeqrt_work(LAPACK_COL_MAJOR, M, N, ib, A, LDA, T, LDT, WORK);
    hqr_shim_tau_from_t(k, ib, T, LDT, TAU);
    return info;
}
static inline int CORE_dtsqrt(int M, int N, int IB, double *A1, int LDA1, double *A2, int LDA2,
                              double *T, int LDT, double *TAU, double *WORK)
{
    int ib = IB < N ? IB : N;
    int info = scipy_LAPACKE_dtpqrt_work(LAPACK_COL_MAJOR, M, N, 0, ib, A1, LDA1, A2, LDA2,
                                         T, LDT, WORK);
    hqr_shim_tau_from_t(N, ib, T, LDT, TAU);
    return info;
}
static inline int CORE_dormqr(int side, int trans, int M, int N, int K, int IB,
                              const double *V, int LDV, const double *T, int LDT,
                              double *C, int LDC, double *WORK, int LDWORK)
{
    (void)LDWORK;
    int ib = IB < K ? IB : K;
    return scipy_LAPACKE_dgemqrt_work(LAPACK_COL_MAJOR, lapack_const(side), lapack_const(trans),
                                      M, N, K, ib, V, LDV, T, LDT, C, LDC, WORK);
}
static inline int CORE_dtsmqr(int side, int trans, int M1, int N1, int M2, int N2, int K, int IB,
                              double *A1, int LDA1, double *A2, int LDA2, const double *V, int LDV,
                              const double *T, int LDT, double *WORK, int LDWORK)
{
    (void)M1; (void)N2; (void)LDWORK;
    int ib = IB < K ? IB : K;
    return scipy_LAPACKE_dtpmqrt_work(LAPACK_COL_MAJOR, lapack_const(side), lapack_const(trans),
                                      M2, N1, K, 0, ib, V, LDV, T, LDT, A1, LDA1, A2, LDA2, WORK);
}
#endif
