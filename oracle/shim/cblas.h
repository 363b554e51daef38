/* CBLAS declarations mapped onto the scipy-bundled OpenBLAS (symbols carry a
 * scipy_ prefix; LP64 integers).  TEST INFRASTRUCTURE ONLY. */
#ifndef HQR_SHIM_CBLAS_H
#define HQR_SHIM_CBLAS_H
typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_ORDER;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
typedef enum { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;
typedef enum { CblasNonUnit = 131, CblasUnit = 132 } CBLAS_DIAG;
typedef enum { CblasLeft = 141, CblasRight = 142 } CBLAS_SIDE;
typedef CBLAS_ORDER CBLAS_LAYOUT;

void scipy_cblas_dcopy(int n, const double *x, int incx, double *y, int incy);
void scipy_cblas_daxpy(int n, double a, const double *x, int incx, double *y, int incy);
void scipy_cblas_dscal(int n, double a, double *x, int incx);
double scipy_cblas_ddot(int n, const double *x, int incx, const double *y, int incy);
double scipy_cblas_dnrm2(int n, const double *x, int incx);
void scipy_cblas_dgemv(CBLAS_ORDER o, CBLAS_TRANSPOSE t, int m, int n, double alpha,
                       const double *a, int lda, const double *x, int incx, double beta,
                       double *y, int incy);
void scipy_cblas_dtrmv(CBLAS_ORDER o, CBLAS_UPLO u, CBLAS_TRANSPOSE t, CBLAS_DIAG d, int n,
                       const double *a, int lda, double *x, int incx);
void scipy_cblas_dger(CBLAS_ORDER o, int m, int n, double alpha, const double *x, int incx,
                      const double *y, int incy, double *a, int lda);
void scipy_cblas_dgemm(CBLAS_ORDER o, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int m, int n,
                       int k, double alpha, const double *a, int lda, const double *b, int ldb,
                       double beta, double *c, int ldc);
void scipy_cblas_dtrmm(CBLAS_ORDER o, CBLAS_SIDE s, CBLAS_UPLO u, CBLAS_TRANSPOSE t,
                       CBLAS_DIAG d, int m, int n, double alpha, const double *a, int lda,
                       double *b, int ldb);
void scipy_openblas_set_num_threads(int n);

#define cblas_dcopy scipy_cblas_dcopy
#define cblas_daxpy scipy_cblas_daxpy
#define cblas_dscal scipy_cblas_dscal
#define cblas_ddot scipy_cblas_ddot
#define cblas_dnrm2 scipy_cblas_dnrm2
#define cblas_dgemv scipy_cblas_dgemv
#define cblas_dtrmv scipy_cblas_dtrmv
#define cblas_dger scipy_cblas_dger
#define cblas_dgemm scipy_cblas_dgemm
#define cblas_dtrmm scipy_cblas_dtrmm
#endif
