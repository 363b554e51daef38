/* LAPACKE work-routine declarations mapped onto the scipy-bundled OpenBLAS.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef HQR_SHIM_LAPACKE_H
#define HQR_SHIM_LAPACKE_H
typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
lapack_int scipy_LAPACKE_dlarft_work(int layout, char direct, char storev, lapack_int n,
                                     lapack_int k, const double *v, lapack_int ldv,
                                     const double *tau, double *t, lapack_int ldt);
lapack_int scipy_LAPACKE_dlarfb_work(int layout, char side, char trans, char direct,
                                     char storev, lapack_int m, lapack_int n, lapack_int k,
                                     const double *v, lapack_int ldv, const double *t,
                                     lapack_int ldt, double *c, lapack_int ldc, double *work,
                                     lapack_int ldwork);
lapack_int scipy_LAPACKE_dgeqrt_work(int layout, lapack_int m, lapack_int n, lapack_int nb,
                                     double *a, lapack_int lda, double *t, lapack_int ldt,
                                     double *work);
lapack_int scipy_LAPACKE_dtpqrt_work(int layout, lapack_int m, lapack_int n, lapack_int l,
                                     lapack_int nb, double *a, lapack_int lda, double *b,
                                     lapack_int ldb, double *t, lapack_int ldt, double *work);
lapack_int scipy_LAPACKE_dgemqrt_work(int layout, char side, char trans, lapack_int m,
                                      lapack_int n, lapack_int k, lapack_int nb,
                                      const double *v, lapack_int ldv, const double *t,
                                      lapack_int ldt, double *c, lapack_int ldc, double *work);
lapack_int scipy_LAPACKE_dtpmqrt_work(int layout, char side, char trans, lapack_int m,
                                      lapack_int n, lapack_int k, lapack_int l, lapack_int nb,
                                      const double *v, lapack_int ldv, const double *t,
                                      lapack_int ldt, double *a, lapack_int lda, double *b,
                                      lapack_int ldb, double *work);
#define LAPACKE_dlarft_work scipy_LAPACKE_dlarft_work
#define LAPACKE_dlarfb_work scipy_LAPACKE_dlarfb_work
#endif
