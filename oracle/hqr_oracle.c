/*
 * hqr_oracle.c -- CPU oracle for the tiled Householder QR path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, calls or
 * executes this file: it is loaded by the tests, by the smoke check and by
 * the CPU-baseline leg of the benchmark, and there only as the checker.
 *
 * It restates, in plain C with no BLAS, the arithmetic that Hybrid3's hot path
 * performs:
 *
 *   - The four PLASMA CORE tile kernels the factorization calls
 *     (Hybrid_tile_QR.c:985 CORE_dgeqrt, :1135 CORE_dtsqrt, :1276 CORE_dormqr,
 *     :1356 CORE_dtsmqr).  PLASMA (comment "PLASMA 2.5.1", Hybrid_make_Q.c:21)
 *     is not vendored in the reference; its published algorithm is restated
 *     here: blocked Householder QR with LAPACK dlarfg reflectors
 *     (beta = -sign(alpha)*||[alpha;x]||, tau = 0 for a trivial reflector),
 *     IB-wide column blocks, and an IB x IB upper-triangular T per block stored
 *     in the LAPACK dgeqrt layout (rows 0..IB-1 of column c hold the T block
 *     that column c belongs to, leading dimension LDT).
 *   - The drivers: Hybrid_tile_QR (flat top-to-bottom TS tree; every tile's
 *     writes are totally ordered by the LIN/MEM dependencies, so a sequential
 *     loop in that order gives the same result as the dynamic schedule),
 *     Hybrid_make_Q (Hybrid_make_Q.c:56-237, full-NB T rebuilt from V/TAU,
 *     V zeroed so that A becomes R), Hybrid_dorgqr (Hybrid_dorgqr.c:22-192),
 *     Hybrid_dormqr (Hybrid_dormqr.c:20-171), Hybrid_dgemm (C = A^T B,
 *     Hybrid_dgemm.c:16-70), Hybrid_make_I (Hybrid_make_I.c:20-53).
 *   - The repo's own tile kernels (tile_kernel.c:19-716) with their own
 *     conventions: beta = +||x||, y_head = alpha - beta, a lower-triangular
 *     full-width T, and their documented quirks.
 *   - The matrix helpers mat_make / mat_remv (glibc rand()/RAND_MAX, filled
 *     column by column, mat_prod.c:157-208) and mat_comp3 (max column
 *     abs-sum, NaN-propagating, mat_prod.c:115-154).
 *
 * Tile layout (mat_prod.h:57-67): tile (i,j) of an MT x NT grid of NB x NB
 * tiles starts at (i + j*MT)*NB*NB and is column-major with ld = NB; the TAU
 * block of tile (i,j) starts at (i + j*MT)*NB.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#include <stdio.h>

#define ORC_EXPORT __attribute__((visibility("default")))

static int imin(int a, int b) { return a < b ? a : b; }

/* Thread count of the oracle's own parallel loops (independent of the
 * OMP_NUM_THREADS list that the reference build needs). */
static int orc_nthreads = 1;
ORC_EXPORT void orc_set_threads(int n) { orc_nthreads = n > 0 ? n : 1; }

/* ---------------------------------------------------------------------------
 * LAPACK-style helpers (restated from LAPACK's published reference algorithms)
 * ------------------------------------------------------------------------- */

/* Euclidean norm with the scaled sum-of-squares recurrence of the LAPACK
 * reference dnrm2, so that it neither overflows nor underflows. */
static double orc_dnrm2(int n, const double *x, int incx)
{
    double scale = 0.0, ssq = 1.0;
    for (int i = 0; i < n; i++) {
        double v = x[(long)i * incx];
        if (v != 0.0) {
            double a = fabs(v);
            if (scale < a) {
                ssq = 1.0 + ssq * (scale / a) * (scale / a);
                scale = a;
            } else {
                ssq += (a / scale) * (a / scale);
            }
        }
    }
    return scale * sqrt(ssq);
}

static double orc_dlapy2(double x, double y)
{
    double xa = fabs(x), ya = fabs(y);
    double w = xa > ya ? xa : ya, z = xa < ya ? xa : ya;
    if (z == 0.0 || w > DBL_MAX) return w;
    return w * sqrt(1.0 + (z / w) * (z / w));
}

/* LAPACK dlarfg: generate H = I - tau*[1;v][1;v]^T with H*[alpha;x] = [beta;0],
 * beta = -sign(alpha)*||[alpha;x]||.  tau = 0 (H = I) when x is zero. */
ORC_EXPORT void orc_dlarfg(int n, double *alpha, double *x, int incx, double *tau)
{
    if (n <= 1) { *tau = 0.0; return; }
    double xnorm = orc_dnrm2(n - 1, x, incx);
    if (xnorm == 0.0) { *tau = 0.0; return; }
    double beta = -copysign(orc_dlapy2(*alpha, xnorm), *alpha);
    const double safmin = DBL_MIN / (DBL_EPSILON * 0.5);
    int knt = 0;
    if (fabs(beta) < safmin) {
        const double rsafmn = 1.0 / safmin;
        do {
            knt++;
            for (int i = 0; i < n - 1; i++) x[(long)i * incx] *= rsafmn;
            beta *= rsafmn;
            *alpha *= rsafmn;
        } while (fabs(beta) < safmin && knt < 20);
        xnorm = orc_dnrm2(n - 1, x, incx);
        beta = -copysign(orc_dlapy2(*alpha, xnorm), *alpha);
    }
    *tau = (beta - *alpha) / beta;
    double s = 1.0 / (*alpha - beta);
    for (int i = 0; i < n - 1; i++) x[(long)i * incx] *= s;
    for (int j = 0; j < knt; j++) beta *= safmin;
    *alpha = beta;
}

/* Apply H^T = I - tau v v^T (v(0) = 1 implicit, v(1:m) = x) from the left to
 * the m x n block C (leading dimension ldc).  LAPACK dlarf, side = 'L'. */
static void orc_apply_reflector(int m, int n, const double *v, double tau,
                                double *C, int ldc)
{
    if (tau == 0.0) return;
    for (int j = 0; j < n; j++) {
        double *c = C + (long)j * ldc;
        double w = c[0];
        for (int r = 1; r < m; r++) w += v[r - 1] * c[r];
        w *= tau;
        c[0] -= w;
        for (int r = 1; r < m; r++) c[r] -= w * v[r - 1];
    }
}

/* LAPACK dgeqr2 on an m x n block: unblocked Householder QR. */
static void orc_dgeqr2(int m, int n, double *A, int lda, double *tau)
{
    int k = imin(m, n);
    for (int i = 0; i < k; i++) {
        double *aii = A + i + (long)i * lda;
        orc_dlarfg(m - i, aii, aii + 1, 1, &tau[i]);
        if (i + 1 < n)
            orc_apply_reflector(m - i, n - i - 1, aii + 1, tau[i],
                                A + i + (long)(i + 1) * lda, lda);
    }
}

/* LAPACK dlarft, direct = 'F', storev = 'C': upper-triangular k x k T with
 * H(0)...H(k-1) = I - V T V^T, V (m x k) unit lower trapezoidal (implicit
 * unit diagonal, entries above it ignored). */
static void orc_dlarft_fc(int m, int k, const double *V, int ldv,
                          const double *tau, double *T, int ldt)
{
    for (int i = 0; i < k; i++) {
        double *ti = T + (long)i * ldt;
        if (tau[i] == 0.0) {
            for (int r = 0; r <= i; r++) ti[r] = 0.0;
            continue;
        }
        /* ti(0:i) = -tau_i * V(i:m, 0:i)^T * v_i, v_i(i) = 1 */
        for (int c = 0; c < i; c++) {
            const double *vc = V + (long)c * ldv;
            const double *vi = V + (long)i * ldv;
            double s = vc[i];
            for (int r = i + 1; r < m; r++) s += vc[r] * vi[r];
            ti[c] = -tau[i] * s;
        }
        /* ti(0:i) = T(0:i,0:i) * ti(0:i), T upper triangular */
        for (int r = 0; r < i; r++) {
            double s = 0.0;
            for (int c = r; c < i; c++) s += T[r + (long)c * ldt] * ti[c];
            ti[r] = s;
        }
        ti[i] = tau[i];
    }
}

/* C (m x n) <- (I - V T V^T)^T C with V m x k unit lower trapezoidal and T
 * k x k upper triangular: LAPACK dlarfb(side='L', trans='T', 'F', 'C'). */
static void orc_dlarfb_lt(int m, int n, int k, const double *V, int ldv,
                          const double *T, int ldt, double *C, int ldc)
{
    double *W = (double *)malloc(sizeof(double) * (size_t)k * (n > 0 ? n : 1));
    for (int j = 0; j < n; j++) {
        const double *c = C + (long)j * ldc;
        for (int a = 0; a < k; a++) {
            const double *va = V + (long)a * ldv;
            double s = c[a];                 /* unit diagonal */
            #pragma omp simd reduction(+:s)
            for (int r = a + 1; r < m; r++) s += va[r] * c[r];
            W[a + (long)j * k] = s;
        }
    }
    /* W <- T^T W */
    for (int j = 0; j < n; j++) {
        double *w = W + (long)j * k;
        for (int a = k - 1; a >= 0; a--) {
            double s = 0.0;
            for (int b = 0; b <= a; b++) s += T[b + (long)a * ldt] * w[b];
            w[a] = s;
        }
    }
    /* C <- C - V W */
    for (int j = 0; j < n; j++) {
        double *c = C + (long)j * ldc;
        const double *w = W + (long)j * k;
        for (int a = 0; a < k; a++) {
            const double *va = V + (long)a * ldv;
            c[a] -= w[a];
            for (int r = a + 1; r < m; r++) c[r] -= va[r] * w[a];
        }
    }
    free(W);
}

/* Triangle-on-square block reflector with l = 0 (the PLASMA "parfb"/"tsrfb"
 * step): [A1(0:k,:); A2] <- (I - [I;V] T [I;V]^T)^T [A1(0:k,:); A2] with V
 * m2 x k dense and T k x k upper triangular. */
static void orc_tsrfb_lt(int k, int n, int m2, double *A1, int lda1,
                         double *A2, int lda2, const double *V, int ldv,
                         const double *T, int ldt)
{
    double *W = (double *)malloc(sizeof(double) * (size_t)k * (n > 0 ? n : 1));
    for (int j = 0; j < n; j++) {
        const double *a1 = A1 + (long)j * lda1;
        const double *a2 = A2 + (long)j * lda2;
        for (int a = 0; a < k; a++) {
            const double *va = V + (long)a * ldv;
            double s = a1[a];
            #pragma omp simd reduction(+:s)
            for (int r = 0; r < m2; r++) s += va[r] * a2[r];
            W[a + (long)j * k] = s;
        }
    }
    for (int j = 0; j < n; j++) {
        double *w = W + (long)j * k;
        for (int a = k - 1; a >= 0; a--) {
            double s = 0.0;
            for (int b = 0; b <= a; b++) s += T[b + (long)a * ldt] * w[b];
            w[a] = s;
        }
    }
    for (int j = 0; j < n; j++) {
        double *a1 = A1 + (long)j * lda1;
        double *a2 = A2 + (long)j * lda2;
        const double *w = W + (long)j * k;
        for (int a = 0; a < k; a++) a1[a] -= w[a];
        for (int a = 0; a < k; a++) {
            const double *va = V + (long)a * ldv;
            for (int r = 0; r < m2; r++) a2[r] -= va[r] * w[a];
        }
    }
    free(W);
}

/* ---------------------------------------------------------------------------
 * PLASMA CORE tile kernels (restated; called at Hybrid_tile_QR.c:985,1135,
 * 1276,1356 and Hybrid_make_Q.c:142,172)
 * ------------------------------------------------------------------------- */

/* CORE_dgeqrt(M,N,IB,A,LDA,T,LDT,TAU,WORK): blocked QR of one tile. */
ORC_EXPORT int orc_core_dgeqrt(int m, int n, int ib, double *A, int lda,
                               double *T, int ldt, double *tau)
{
    if (m < 0 || n < 0 || ib < 0 || lda < (m > 1 ? m : 1)) return -1;
    int k = imin(m, n);
    for (int i = 0; i < k; i += ib) {
        int sb = imin(ib, k - i);
        double *aii = A + i + (long)i * lda;
        orc_dgeqr2(m - i, sb, aii, lda, tau + i);
        orc_dlarft_fc(m - i, sb, aii, lda, tau + i, T + (long)i * ldt, ldt);
        if (n > i + sb)
            orc_dlarfb_lt(m - i, n - i - sb, sb, aii, lda, T + (long)i * ldt, ldt,
                          A + i + (long)(i + sb) * lda, lda);
    }
    return 0;
}

/* CORE_dtsmqr(Left, Trans, M1,N1,M2,N2,K,IB, A1,LDA1, A2,LDA2, V,LDV, T,LDT):
 * apply the transpose of the block reflector of a TSQRT to [A1; A2]. */
ORC_EXPORT int orc_core_dtsmqr(int m1, int n1, int m2, int n2, int k, int ib,
                               double *A1, int lda1, double *A2, int lda2,
                               const double *V, int ldv, const double *T, int ldt)
{
    if (n1 != n2 || k > m1) return -1;
    for (int i = 0; i < k; i += ib) {
        int kb = imin(ib, k - i);
        orc_tsrfb_lt(kb, n1, m2, A1 + i, lda1, A2, lda2,
                     V + (long)i * ldv, ldv, T + (long)i * ldt, ldt);
    }
    return 0;
}

/* CORE_dtsqrt(M,N,IB,A1,LDA1,A2,LDA2,T,LDT,TAU,WORK): QR of the stacked pair
 * [R; A2], R = A1 upper triangular N x N, A2 dense M x N.  A2 becomes V. */
ORC_EXPORT int orc_core_dtsqrt(int m, int n, int ib, double *A1, int lda1,
                               double *A2, int lda2, double *T, int ldt,
                               double *tau)
{
    if (m < 0 || n < 0) return -1;
    double *work = (double *)malloc(sizeof(double) * (size_t)(ib > 0 ? ib : 1));
    for (int ii = 0; ii < n; ii += ib) {
        int sb = imin(n - ii, ib);
        for (int i = 0; i < sb; i++) {
            int c = ii + i;
            double *v = A2 + (long)c * lda2;
            orc_dlarfg(m + 1, A1 + c + (long)c * lda1, v, 1, &tau[c]);
            /* apply H(c) to the rest of this column block */
            int nr = sb - i - 1;
            if (nr > 0 && c + 1 < n) {
                for (int j = 0; j < nr; j++) {
                    int cj = c + 1 + j;
                    double w = A1[c + (long)cj * lda1];
                    const double *a2 = A2 + (long)cj * lda2;
                    for (int r = 0; r < m; r++) w += a2[r] * v[r];
                    work[j] = w;
                }
                double alpha = -tau[c];
                for (int j = 0; j < nr; j++) {
                    int cj = c + 1 + j;
                    A1[c + (long)cj * lda1] += alpha * work[j];
                    double *a2 = A2 + (long)cj * lda2;
                    for (int r = 0; r < m; r++) a2[r] += alpha * v[r] * work[j];
                }
            }
            /* T(0:i, c) = -tau_c * V(:, ii:c)^T v_c, then T(0:i,c) = Tblk * T(0:i,c) */
            double *tc = T + (long)c * ldt;
            for (int a = 0; a < i; a++) {
                const double *va = A2 + (long)(ii + a) * lda2;
                double s = 0.0;
                for (int r = 0; r < m; r++) s += va[r] * v[r];
                tc[a] = -tau[c] * s;
            }
            for (int r = 0; r < i; r++) {
                double s = 0.0;
                for (int a = r; a < i; a++) s += T[r + (long)(ii + a) * ldt] * tc[a];
                tc[r] = s;
            }
            tc[i] = tau[c];
        }
        if (n > ii + sb) {
            orc_core_dtsmqr(sb, n - (ii + sb), m, n - (ii + sb), sb, ib,
                            A1 + ii + (long)(ii + sb) * lda1, lda1,
                            A2 + (long)(ii + sb) * lda2, lda2,
                            A2 + (long)ii * lda2, lda2, T + (long)ii * ldt, ldt);
        }
    }
    free(work);
    return 0;
}

/* CORE_dormqr(Left, Trans, M,N,K,IB, V,LDV, T,LDT, C,LDC): C <- Q^T C for the
 * Q of a GEQRT tile (V unit lower, implicit diagonal). */
ORC_EXPORT int orc_core_dormqr(int m, int n, int k, int ib, const double *V,
                               int ldv, const double *T, int ldt, double *C,
                               int ldc)
{
    if (k > m) return -1;
    for (int i = 0; i < k; i += ib) {
        int kb = imin(ib, k - i);
        orc_dlarfb_lt(m - i, n, kb, V + i + (long)i * ldv, ldv,
                      T + (long)i * ldt, ldt, C + i, ldc);
    }
    return 0;
}

/* crayj_dtsrft (Hybrid_make_Q.c:14-44): IB-blocked upper T of a TS tile from
 * V (M x N dense) and TAU.  With IB = N it is the full N x N T. */
ORC_EXPORT void orc_dtsrft(int m, int n, int ib, const double *V, int ldv,
                           const double *tau, double *T, int ldt)
{
    for (int ii = 0; ii < n; ii += ib) {
        int sb = imin(n - ii, ib);
        for (int i = 0; i < sb; i++) {
            double *tc = T + (long)(ii + i) * ldt;
            const double *vi = V + (long)(ii + i) * ldv;
            for (int a = 0; a < i; a++) {
                const double *va = V + (long)(ii + a) * ldv;
                double s = 0.0;
                for (int r = 0; r < m; r++) s += va[r] * vi[r];
                tc[a] = -tau[ii + i] * s;
            }
            for (int r = 0; r < i; r++) {
                double s = 0.0;
                for (int a = r; a < i; a++) s += T[r + (long)(ii + a) * ldt] * tc[a];
                tc[r] = s;
            }
            tc[i] = tau[ii + i];
        }
    }
}

/* Full upper T (direct 'F', storev 'C') of a GEQRT tile: LAPACKE_dlarft_work
 * as called at Hybrid_make_Q.c:124-130. */
ORC_EXPORT void orc_dlarft(int m, int k, const double *V, int ldv,
                           const double *tau, double *T, int ldt)
{
    orc_dlarft_fc(m, k, V, ldv, tau, T, ldt);
}

/* ---------------------------------------------------------------------------
 * Drivers
 * ------------------------------------------------------------------------- */

#define TILE(P, i, j) ((P) + ((long)(i) + (long)(j) * MT) * (long)NB * NB)
#define TAUP(P, i, j) ((P) + ((long)(i) + (long)(j) * MT) * (long)NB)

/* Hybrid_tile_QR (Hybrid_tile_QR.c:307-1589) with one rank.  The tasks are run
 * in a sequential order that respects every LIN/MEM/YTM edge of the
 * reference's dependency table (Hybrid_tile_QR.c:515-580); because each tile's
 * updates are totally ordered by those edges, the result equals the dynamic
 * schedule's.  The step count is min(MT, NT); unlike the reference, a tall
 * matrix (MT > NT) terminates (the reference only stops at a GEQRT on the last
 * tile row, Hybrid_tile_QR.c:1008,1037-1040).  If Tout is non-NULL it receives
 * each panel tile's IB-blocked T (ldt = NB), in the same tile layout as A. */
ORC_EXPORT int orc_tile_qr(long M, long N, int NB, int IB, double *A, double *TAU,
                           double *Tout)
{
    int MT = (int)(M / NB), NT = (int)(N / NB);
    int steps = imin(MT, NT);
    double *Tt = (double *)calloc((size_t)NB * NB, sizeof(double));
    for (int i = 0; i < steps; i++) {
        /* GEQRT(i,i,i) then the LARFB(i,j,i) row */
        memset(Tt, 0, sizeof(double) * (size_t)NB * NB);
        orc_core_dgeqrt(NB, NB, IB, TILE(A, i, i), NB, Tt, NB, TAUP(TAU, i, i));
        if (Tout) memcpy(TILE(Tout, i, i), Tt, sizeof(double) * (size_t)NB * NB);
        #pragma omp parallel for schedule(dynamic) num_threads(orc_nthreads)
        for (int j = i + 1; j < NT; j++)
            orc_core_dormqr(NB, NB, NB, IB, TILE(A, i, i), NB, Tt, NB, TILE(A, i, j), NB);
        /* TSQRT(i,i,k) then the SSRFB(i,j,k) row, k = i+1..MT-1 */
        for (int k = i + 1; k < MT; k++) {
            memset(Tt, 0, sizeof(double) * (size_t)NB * NB);
            orc_core_dtsqrt(NB, NB, IB, TILE(A, i, i), NB, TILE(A, k, i), NB, Tt, NB,
                            TAUP(TAU, k, i));
            if (Tout) memcpy(TILE(Tout, k, i), Tt, sizeof(double) * (size_t)NB * NB);
            #pragma omp parallel for schedule(dynamic) num_threads(orc_nthreads)
            for (int j = i + 1; j < NT; j++)
                orc_core_dtsmqr(NB, NB, NB, NB, NB, IB, TILE(A, i, j), NB, TILE(A, k, j), NB,
                                TILE(A, k, i), NB, Tt, NB);
        }
    }
    free(Tt);
    return 0;
}

/* Hybrid_make_Q (Hybrid_make_Q.c:56-237) with one rank: Q (caller-zeroed, same
 * tile grid as RY) receives Q^T = H_last^T ... H_1^T applied to I; full-NB T
 * factors are rebuilt from V and TAU; V is zeroed so that RY becomes R. */
ORC_EXPORT void orc_make_Q(long M, long N, int NB, double *Q, double *RY, double *TAU)
{
    int MT = (int)(M / NB), NT = (int)(N / NB);
    double *Y = (double *)calloc((size_t)NB * NB, sizeof(double));
    double *T = (double *)calloc((size_t)NB * NB, sizeof(double));
    for (int c = 0; c < NT; c++) {
        double *q = TILE(Q, c, c);
        for (int r = 0; r < NB; r++) q[r + (long)r * NB] = 1.0;
    }
    int steps = imin(MT, NT);
    for (int gi = 0; gi < steps; gi++) {
        double *ry = TILE(RY, gi, gi);
        for (int ii = 0; ii < NB - 1; ii++) {
            for (int r = ii + 1; r < NB; r++) Y[r + (long)ii * NB] = ry[r + (long)ii * NB];
            Y[ii + (long)ii * NB] = 1.0;
        }
        Y[(long)NB * NB - 1] = 0.0;
        orc_dlarft_fc(NB, NB, Y, NB, TAUP(TAU, gi, gi), T, NB);
        #pragma omp parallel for schedule(dynamic) num_threads(orc_nthreads)
        for (int j = 0; j < NT; j++)
            orc_core_dormqr(NB, NB, NB, NB, Y, NB, T, NB, TILE(Q, gi, j), NB);
        for (int c = 0; c < NB; c++)
            for (int r = c + 1; r < NB; r++) ry[r + (long)c * NB] = 0.0;
        for (int k = gi + 1; k < MT; k++) {
            double *v = TILE(RY, k, gi);
            orc_dtsrft(NB, NB, NB, v, NB, TAUP(TAU, k, gi), T, NB);
            #pragma omp parallel for schedule(dynamic) num_threads(orc_nthreads)
            for (int j = 0; j < NT; j++)
                orc_core_dtsmqr(NB, NB, NB, NB, NB, NB, TILE(Q, gi, j), NB, TILE(Q, k, j), NB,
                                v, NB, T, NB);
            memset(v, 0, sizeof(double) * (size_t)NB * NB);
        }
    }
    free(Y);
    free(T);
}

/* Hybrid_make_I (Hybrid_make_I.c:20-53): zero the whole array, unit diagonal. */
ORC_EXPORT void orc_make_I(long M, long N, int NB, double *Id)
{
    int MT = (int)(M / NB), NT = (int)(N / NB);
    memset(Id, 0, sizeof(double) * (size_t)M * (size_t)N);
    for (int c = 0; c < NT; c++) {
        double *q = TILE(Id, c, c);
        (void)MT;
        for (int r = 0; r < NB; r++) q[r + (long)r * NB] = 1.0;
    }
}

/* Hybrid_dgemm (Hybrid_dgemm.c:16-70): tile-wise C = A^T B. */
ORC_EXPORT void orc_dgemm_tn(long M, long N, int NB, const double *A,
                             const double *B, double *C)
{
    int MT = (int)(M / NB), NT = (int)(N / NB);
    #pragma omp parallel for collapse(2) schedule(dynamic) num_threads(orc_nthreads)
    for (int i = 0; i < NT; i++) {
        for (int j = 0; j < NT; j++) {
            if (i >= MT) continue;
            double *c = TILE(C, i, j);
            memset(c, 0, sizeof(double) * (size_t)NB * NB);
            for (int k = 0; k < MT; k++) {
                const double *a = TILE(A, k, i);
                const double *b = TILE(B, k, j);
                for (int cc = 0; cc < NB; cc++)
                    for (int rr = 0; rr < NB; rr++) {
                        double s = 0.0;
                        const double *ar = a + (long)rr * NB, *bc = b + (long)cc * NB;
                        for (int t = 0; t < NB; t++) s += ar[t] * bc[t];
                        c[rr + (long)cc * NB] += s;
                    }
            }
        }
    }
}

/* mat_make / mat_remv (mat_prod.c:157-208): glibc rand()/RAND_MAX in the
 * (tile column, column, tile row, row) order, seed + rank; sign = +1 makes,
 * sign = -1 subtracts. */
ORC_EXPORT void orc_mat_fill(long M, long N, int NB, double *A, unsigned seed,
                             int subtract)
{
    int MT = (int)(M / NB), NT = (int)(N / NB);
    srand(seed);
    for (int j = 0; j < NT; j++)
        for (int jj = 0; jj < NB; jj++)
            for (int i = 0; i < MT; i++)
                for (int ii = 0; ii < NB; ii++) {
                    double n = (double)rand() / (double)RAND_MAX;
                    double *p = TILE(A, i, j) + ii + (long)jj * NB;
                    if (subtract) *p -= n; else *p = n;
                }
}

/* mat_comp3 (mat_prod.c:115-154): max over columns of the column abs-sum of a
 * column-major M x N array; a NaN column sum is returned at once. */
ORC_EXPORT double orc_mat_comp3(long M, long N, const double *E)
{
    double e = 0.0;
    for (long i = 0; i < N; i++) {
        double s = 0.0;
        for (long j = 0; j < M; j++) s += fabs(E[i * M + j]);
        if (s > e) e = s;
        if (isnan(s)) { e = s; break; }
    }
    return e;
}

/* mat_dprint (mat_prod.c:260-281): tile layout -> column-major M x N. */
ORC_EXPORT void orc_tile_to_colmajor(long M, long N, int NB, const double *tiles,
                                     double *out)
{
    int MT = (int)(M / NB), NT = (int)(N / NB);
    long c = 0;
    for (int j = 0; j < NT; j++)
        for (int l = 0; l < NB; l++)
            for (int i = 0; i < MT; i++)
                for (int k = 0; k < NB; k++)
                    out[c++] = TILE(tiles, i, j)[k + (long)l * NB];
}

/* ---------------------------------------------------------------------------
 * The repo's own tile kernels (tile_kernel.c), restated with their own
 * conventions: beta = +||x||, y_head = alpha - beta, TAU = t*y_head^2 with
 * t = 2/(y_head^2 + ||x||^2), V scaled by 1/y_head; T lower triangular with
 * T(i,i) = tau_i and T(i,0:i) = -tau_i (T(0:i,0:i)^T (Y^T y_i)(0:i)).
 * ------------------------------------------------------------------------- */

/* tile_sub_dgeqr2 (tile_kernel.c:138-218).  Quirks kept: no zero-norm guard
 * (x = 0 with alpha > 0 divides by zero); with row == col the last TAU is left
 * unwritten and Y(col-1,col-1) is set to 0. */
ORC_EXPORT void orc_tk_sub_dgeqr2(int row, int col, double *A, int lda,
                                  double *TAU, double *Y, double *work)
{
    double *yA = work;
    int i;
    for (i = 0; i < col - 1; i++) {
        double *aii = A + i + (long)lda * i;
        /* yA(0:col-i) = A(i+1:row, i)^T A(i+1:row, i:col) */
        for (int c = 0; c < col - i; c++) {
            const double *ac = A + i + 1 + (long)lda * (i + c);
            double s = 0.0;
            for (int r = 0; r < row - i - 1; r++) s += aii[1 + r] * ac[r];
            yA[c] = s;
        }
        double a_head = *aii;
        double norm_1 = yA[0];
        double norm = norm_1 + a_head * a_head;
        double b = sqrt(norm);
        double y_head = a_head - b;
        *aii = y_head;
        double t = 2.0 / (y_head * y_head + norm_1);
        for (int c = 0; c < col - i - 1; c++) yA[1 + c] += y_head * A[i + (long)lda * (i + 1 + c)];
        for (int c = 0; c < col - i - 1; c++) {
            double *ac = A + i + (long)lda * (i + 1 + c);
            for (int r = 0; r < row - i; r++) ac[r] += -t * aii[r] * yA[1 + c];
        }
        *aii = b;
        for (int r = 0; r < row - i - 1; r++) aii[1 + r] *= 1.0 / y_head;
        for (int r = 0; r < row - i - 1; r++) Y[i + (long)lda * i + 1 + r] = aii[1 + r];
        Y[i + (long)lda * i] = 1.0;
        TAU[i] = t * y_head * y_head;
    }
    if (row > col) {
        i = col - 1;
        double *aii = A + i + (long)lda * i;
        double s = 0.0;
        for (int r = 0; r < row - i - 1; r++) s += aii[1 + r] * aii[1 + r];
        double a_head = *aii;
        double norm_1 = s;
        double norm = norm_1 + a_head * a_head;
        double b = sqrt(norm);
        double y_head = a_head - b;
        *aii = b;
        for (int r = 0; r < row - i - 1; r++) aii[1 + r] *= 1.0 / y_head;
        for (int r = 0; r < row - i - 1; r++) Y[i + (long)lda * i + 1 + r] = aii[1 + r];
        Y[i + (long)lda * i] = 1.0;
        double t = 2.0 / (y_head * y_head + norm_1);
        TAU[i] = t * y_head * y_head;
    } else if (row == col) {
        Y[i + (long)lda * i] = 0.0;
    }
}

/* tile_sub_dlarft (tile_kernel.c:220-262): lower-triangular T. */
ORC_EXPORT void orc_tk_sub_dlarft(int row, int col, const double *Y, int lda,
                                  const double *TAU, double *T, int ldt,
                                  double *work)
{
    double *YtY = work;                       /* col x col, ld = col */
    for (int a = 0; a < col; a++)
        for (int b = 0; b < col; b++) {
            double s = 0.0;
            for (int r = 0; r < row; r++) s += Y[r + (long)a * lda] * Y[r + (long)b * lda];
            YtY[a + (long)b * col] = s;
        }
    for (int i = 0; i < col; i++) T[i + (long)i * ldt] = TAU[i];
    for (int i = 1; i < col; i++) {
        double alpha = -T[i + (long)i * ldt];
        /* T(i, r) = alpha * sum_c T(c, r) * YtY(i, c) for r < i (T lower) */
        double tmp[1024];
        double *dst = i <= 1024 ? tmp : (double *)malloc(sizeof(double) * i);
        for (int r = 0; r < i; r++) {
            double s = 0.0;
            for (int c = 0; c < i; c++) s += T[c + (long)r * ldt] * YtY[i + (long)c * col];
            dst[r] = alpha * s;
        }
        for (int r = 0; r < i; r++) T[i + (long)r * ldt] = dst[r];
        if (dst != tmp) free(dst);
    }
}

/* tile_sub_dlarfb (tile_kernel.c:264-311): A <- (I - Y T Y^T) A with Y an
 * explicit row x row lower-triangular matrix (its diagonal is used as stored)
 * and T lower triangular Y_col x Y_col. */
ORC_EXPORT void orc_tk_sub_dlarfb(int row, int Y_col, int A_col, const double *Y,
                                  int ldy, const double *T, int ldt, double *A,
                                  int lda, double *work)
{
    double *D = work;                          /* row x A_col, ld = row */
    for (int c = 0; c < A_col; c++)
        for (int r = 0; r < Y_col; r++) {
            /* (Y^T A)(r, c) with Y lower: sum over q >= r.  Rows >= Y_col of
             * the reference's product are computed there but never used. */
            double s = 0.0;
            for (int q = r; q < row; q++) s += Y[q + (long)r * ldy] * A[q + (long)c * lda];
            D[r + (long)c * row] = s;
        }
    for (int c = 0; c < A_col; c++) {
        double *d = D + (long)c * row;
        for (int r = Y_col - 1; r >= 0; r--) {
            double s = 0.0;
            for (int q = 0; q <= r; q++) s += T[r + (long)q * ldt] * d[q];
            d[r] = s;
        }
    }
    for (int c = 0; c < A_col; c++)
        for (int r = 0; r < row; r++) {
            double s = 0.0;
            for (int q = 0; q < Y_col; q++) s += Y[r + (long)q * ldy] * D[q + (long)c * row];
            A[r + (long)c * lda] -= s;
        }
}

/* tile_sub_dssrfb (tile_kernel.c:313-363). */
ORC_EXPORT void orc_tk_sub_dssrfb(int over_row, int under_row, int Y_col, int A_col,
                                  const double *Y, int ldy, const double *T, int ldt,
                                  double *A1, int lda1, double *A2, int lda2,
                                  double *work)
{
    double *D = work;                          /* over_row x A_col, ld = over_row */
    int ld1 = over_row;
    for (int c = 0; c < A_col; c++)
        for (int r = 0; r < over_row; r++) D[r + (long)c * ld1] = A1[r + (long)c * lda1];
    for (int c = 0; c < A_col; c++)
        for (int r = 0; r < Y_col; r++) {
            double s = 0.0;
            for (int q = 0; q < under_row; q++) s += Y[q + (long)r * ldy] * A2[q + (long)c * lda2];
            D[r + (long)c * ld1] += s;
        }
    for (int c = 0; c < A_col; c++) {
        double *d = D + (long)c * ld1;
        for (int r = Y_col - 1; r >= 0; r--) {
            double s = 0.0;
            for (int q = 0; q <= r; q++) s += T[r + (long)q * ldt] * d[q];
            d[r] = s;
        }
    }
    for (int c = 0; c < A_col; c++)
        for (int r = 0; r < over_row; r++) A1[r + (long)c * lda1] -= D[r + (long)c * ld1];
    for (int c = 0; c < A_col; c++)
        for (int r = 0; r < under_row; r++) {
            double s = 0.0;
            for (int q = 0; q < Y_col; q++) s += Y[r + (long)q * ldy] * D[q + (long)c * ld1];
            A2[r + (long)c * lda2] -= s;
        }
}

/* tile_sub_dtsqr2 (tile_kernel.c:654-716): unblocked TS QR of [A1; A2] with the
 * repo's beta = +||x|| convention and no zero-norm guard. */
ORC_EXPORT void orc_tk_sub_dtsqr2(int row, int col, double *A1, int lda1,
                                  double *A2, int lda2, double *TAU, double *work)
{
    double *dv = work;
    int i;
    for (i = 0; i < col - 1; i++) {
        double *v = A2 + (long)i * lda2;
        for (int c = 0; c < col - i; c++) {
            const double *ac = A2 + (long)(i + c) * lda2;
            double s = 0.0;
            for (int r = 0; r < row; r++) s += v[r] * ac[r];
            dv[c] = s;
        }
        double a_head = A1[i + (long)i * lda1];
        double norm_1 = dv[0];
        double norm = norm_1 + a_head * a_head;
        double b = sqrt(norm);
        double y_head = a_head - b;
        double t = 2.0 / (y_head * y_head + norm_1);
        for (int c = 0; c < col - i - 1; c++) dv[1 + c] += y_head * A1[i + (long)(i + 1 + c) * lda1];
        for (int c = 0; c < col - i - 1; c++) A1[i + (long)(i + 1 + c) * lda1] += -t * y_head * dv[1 + c];
        for (int c = 0; c < col - i - 1; c++) {
            double *ac = A2 + (long)(i + 1 + c) * lda2;
            for (int r = 0; r < row; r++) ac[r] += -t * v[r] * dv[1 + c];
        }
        A1[i + (long)i * lda1] = b;
        for (int r = 0; r < row; r++) v[r] *= 1.0 / y_head;
        TAU[i] = t * y_head * y_head;
    }
    double *v = A2 + (long)i * lda2;
    double s = 0.0;
    for (int r = 0; r < row; r++) s += v[r] * v[r];
    double a_head = A1[i + (long)i * lda1];
    double norm_1 = s;
    double norm = norm_1 + a_head * a_head;
    double b = sqrt(norm);
    double y_head = a_head - b;
    double t = 2.0 / (y_head * y_head + norm_1);
    A1[i + (long)i * lda1] = b;
    for (int r = 0; r < row; r++) v[r] *= 1.0 / y_head;
    TAU[i] = t * y_head * y_head;
}

/* tile_dgeqrt (tile_kernel.c:28-57).  Quirk kept: only the diagonal T blocks
 * are built (no coupling between blocks). */
ORC_EXPORT void orc_tk_dgeqrt(int row, int col, int block, double *A, int lda,
                              double *TAU, double *Y, double *T, int ldt,
                              double *work)
{
    int i;
    for (i = 0; i < col - block; i += block) {
        orc_tk_sub_dgeqr2(row - i, block, A + i * lda + i, lda, TAU + i, Y + i * lda + i, work);
        orc_tk_sub_dlarft(row - i, block, Y + i * lda + i, lda, TAU + i, T + i * ldt + i, ldt, work);
        orc_tk_sub_dlarfb(row - i, block, col - i - block, Y + i * lda + i, lda,
                          T + i * ldt + i, ldt, A + (i + block) * lda + i, lda, work);
    }
    orc_tk_sub_dgeqr2(row - i, col - i, A + i * lda + i, lda, TAU + i, Y + i * lda + i, work);
    orc_tk_sub_dlarft(row - i, col - i, Y + i * lda + i, lda, TAU + i, T + i * ldt + i, ldt, work);
}

/* tile_dtsqrt (tile_kernel.c:60-104). */
ORC_EXPORT void orc_tk_dtsqrt(int row, int col, int block, double *A1, int lda1,
                              double *A2, int lda2, double *TAU, double *T, int ldt,
                              double *work)
{
    int i;
    for (i = 0; i < col - block; i += block) {
        orc_tk_sub_dtsqr2(row, block, A1 + i + i * lda1, lda1, A2 + i * lda2, lda2, TAU + i, work);
        orc_tk_sub_dlarft(row, block, A2 + i * lda2, lda2, TAU + i, T + i * ldt + i, ldt, work);
        orc_tk_sub_dssrfb(block, row, block, col - i - block, A2 + i * lda2, lda2,
                          T + i + i * ldt, ldt, A1 + i + (i + block) * lda1, lda1,
                          A2 + (i + block) * lda2, lda2, work);
    }
    if (col % block > 0) {
        i = block * (col / block);
        orc_tk_sub_dtsqr2(row, col % block, A1 + i + i * lda1, lda1, A2 + i * lda2, lda2, TAU + i, work);
        orc_tk_sub_dlarft(row, col % block, A2 + i * lda2, lda2, TAU + i, T + i * ldt + i, ldt, work);
    } else {
        i = col - block;
        orc_tk_sub_dtsqr2(row, block, A1 + i + i * lda1, lda1, A2 + i * lda2, lda2, TAU + i, work);
        orc_tk_sub_dlarft(row, block, A2 + i * lda2, lda2, TAU + i, T + i * ldt + i, ldt, work);
    }
}

/* tile_dlarft (tile_kernel.c:368-437).  block < 2 builds the full lower T;
 * 2 <= block < col builds only the off-diagonal coupling blocks from the
 * existing diagonal blocks; block >= col leaves T untouched (quirk kept). */
ORC_EXPORT void orc_tk_dlarft(int row, int col, int block, const double *Y, int lda,
                              const double *TAU, double *T, int ldt, double *work)
{
    if (block < 2) {
        orc_tk_sub_dlarft(row, col, Y, lda, TAU, T, ldt, work);
        return;
    }
    if (block >= col) return;
    int ldyty = (col / block) * block + block;
    double *YtY = work;                   /* row-major col x col, ld = ldyty */
    double *T1 = work + (long)row * col;   /* i x block, row-major, ld = block */
    /* Row-major C(a,b) = sum_r Y(a,r) Y(b,r) with Y viewed row-major ld = lda:
     * Yrm(a, r) = Y[a*lda + r]. */
    for (int a = 0; a < col; a++)
        for (int b = 0; b < col; b++) {
            double s = 0.0;
            for (int r = 0; r < row; r++) s += Y[(long)a * lda + r] * Y[(long)b * lda + r];
            YtY[(long)a * ldyty + b] = s;
        }
    for (int i = block; i < col - block; i += block) {
        /* T1(0:i, 0:block) = Trm(0:i, 0:i) * YtYrm(0:i, i:i+block); Trm(a,b) = T[a*ldt+b] */
        for (int a = 0; a < i; a++)
            for (int b = 0; b < block; b++) {
                double s = 0.0;
                for (int q = 0; q < i; q++) s += T[(long)a * ldt + q] * YtY[(long)q * ldyty + i + b];
                T1[(long)a * block + b] = s;
            }
        /* Trm(0:i, i:i+block) = -T1 * Trm(i:i+block, i:i+block) */
        for (int a = 0; a < i; a++)
            for (int b = 0; b < block; b++) {
                double s = 0.0;
                for (int q = 0; q < block; q++) s += T1[(long)a * block + q] * T[(long)(i + q) * ldt + i + b];
                T[(long)a * ldt + i + b] = -s;
            }
    }
    for (int i = (col / block) * block; i < col; i++) {
        double alpha = -T[i + (long)i * ldt];
        double tmp[1024];
        double *dst = i <= 1024 ? tmp : (double *)malloc(sizeof(double) * (i > 0 ? i : 1));
        for (int a = 0; a < i; a++) {
            double s = 0.0;
            for (int q = 0; q < i; q++) s += T[(long)a * ldt + q] * YtY[(long)q * ldyty + i];
            dst[a] = alpha * s;
        }
        for (int a = 0; a < i; a++) T[(long)a * ldt + i] = dst[a];
        if (dst != tmp) free(dst);
    }
}

/* Hybrid_dorgqr (Hybrid_dorgqr.c:22-192) with one rank: Q <- Q^T of the
 * factorization, built with the repo's own lower-T tile kernels; V is kept. */
ORC_EXPORT void orc_dorgqr(long M, long N, int NB, double *Q, double *RY, double *TAU)
{
    int MT = (int)(M / NB), NT = (int)(N / NB);
    double *Y = (double *)calloc((size_t)NB * NB, sizeof(double));
    double *T = (double *)calloc((size_t)NB * NB, sizeof(double));
    orc_make_I(M, N, NB, Q);
    int steps = imin(MT, NT);
    for (int gi = 0; gi < steps; gi++) {
        double *ry = TILE(RY, gi, gi);
        for (int ii = 0; ii < NB - 1; ii++) {
            for (int r = ii + 1; r < NB; r++) Y[r + (long)ii * NB] = ry[r + (long)ii * NB];
            Y[ii + (long)ii * NB] = 1.0;
        }
        Y[(long)NB * NB - 1] = 0.0;
        double *work = (double *)calloc((size_t)3 * NB * NB, sizeof(double));
        orc_tk_dlarft(NB, NB, 1, Y, NB, TAUP(TAU, gi, gi), T, NB, work);
        free(work);
        #pragma omp parallel for schedule(dynamic) num_threads(orc_nthreads)
        for (int j = 0; j < NT; j++) {
            double *w = (double *)malloc(sizeof(double) * 3 * (size_t)NB * NB);
            orc_tk_sub_dlarfb(NB, NB, NB, Y, NB, T, NB, TILE(Q, gi, j), NB, w);
            free(w);
        }
        for (int k = gi + 1; k < MT; k++) {
            double *v = TILE(RY, k, gi);
            work = (double *)calloc((size_t)3 * NB * NB, sizeof(double));
            orc_tk_dlarft(NB, NB, 1, v, NB, TAUP(TAU, k, gi), T, NB, work);
            free(work);
            #pragma omp parallel for schedule(dynamic) num_threads(orc_nthreads)
            for (int j = 0; j < NT; j++) {
                double *w = (double *)malloc(sizeof(double) * 3 * (size_t)NB * NB);
                orc_tk_sub_dssrfb(NB, NB, NB, NB, v, NB, T, NB, TILE(Q, gi, j), NB,
                                  TILE(Q, k, j), NB, w);
                free(w);
            }
        }
    }
    free(Y);
    free(T);
}

/* Hybrid_dormqr (Hybrid_dormqr.c:20-171) with one rank: C <- Q^T C, C in a
 * tile grid with the same NB and MT as RY and its own tile-column count CT
 * (the reference uses RY's own grid, CT = NT). */
ORC_EXPORT void orc_dormqr(long M, long N, int NB, const double *RY, const double *TAU,
                           double *C, int CT)
{
    int MT = (int)(M / NB), NT = (int)(N / NB);
    double *Y = (double *)calloc((size_t)NB * NB, sizeof(double));
    double *T = (double *)calloc((size_t)NB * NB, sizeof(double));
    int steps = imin(MT, NT);
    for (int gi = 0; gi < steps; gi++) {
        const double *ry = TILE(RY, gi, gi);
        for (int ii = 0; ii < NB - 1; ii++) {
            for (int r = ii + 1; r < NB; r++) Y[r + (long)ii * NB] = ry[r + (long)ii * NB];
            Y[ii + (long)ii * NB] = 1.0;
        }
        Y[(long)NB * NB - 1] = 0.0;
        double *work = (double *)calloc((size_t)3 * NB * NB, sizeof(double));
        orc_tk_dlarft(NB, NB, 1, Y, NB, TAUP(TAU, gi, gi), T, NB, work);
        free(work);
        #pragma omp parallel for schedule(dynamic) num_threads(orc_nthreads)
        for (int j = 0; j < CT; j++) {
            double *w = (double *)malloc(sizeof(double) * 3 * (size_t)NB * NB);
            orc_tk_sub_dlarfb(NB, NB, NB, Y, NB, T, NB, TILE(C, gi, j), NB, w);
            free(w);
        }
        for (int k = gi + 1; k < MT; k++) {
            const double *v = TILE(RY, k, gi);
            work = (double *)calloc((size_t)3 * NB * NB, sizeof(double));
            orc_tk_dlarft(NB, NB, 1, v, NB, TAUP(TAU, k, gi), T, NB, work);
            free(work);
            #pragma omp parallel for schedule(dynamic) num_threads(orc_nthreads)
            for (int j = 0; j < CT; j++) {
                double *w = (double *)malloc(sizeof(double) * 3 * (size_t)NB * NB);
                orc_tk_sub_dssrfb(NB, NB, NB, NB, v, NB, T, NB, TILE(C, gi, j), NB,
                                  TILE(C, k, j), NB, w);
                free(w);
            }
        }
    }
    free(Y);
    free(T);
}

/* ---------------------------------------------------------------------------
 * Task-parallel drivers (the CPU baseline).  The same tile kernels as above,
 * scheduled like the reference's dynamic DAG (Hybrid_tile_QR.c:905-1461):
 * OpenMP task dependences on tiles stand for its MEM/LIN/YTM bits, and the
 * GEQRT tile is copied for its LARFB row (the reference's glob_YT copy,
 * Hybrid_tile_QR.c:1066-1071) so that the TS chain does not wait for that row.
 * ------------------------------------------------------------------------- */
ORC_EXPORT int orc_tile_qr_dag(long M, long N, int NB, int IB, double *A, double *TAU)
{
    int MT = (int)(M / NB), NT = (int)(N / NB);
    int steps = imin(MT, NT);
    const size_t t2 = (size_t)NB * NB;
    double *Tall = (double *)calloc((size_t)M * (size_t)N, sizeof(double));
    double *Ycopy = (double *)calloc((size_t)steps * t2, sizeof(double));
    double *Tcopy = (double *)calloc((size_t)steps * t2, sizeof(double));
    if (!Tall || !Ycopy || !Tcopy) { free(Tall); free(Ycopy); free(Tcopy); return -1; }
    #pragma omp parallel num_threads(orc_nthreads)
    #pragma omp single
    for (int i = 0; i < steps; i++) {
        double *aii = TILE(A, i, i), *tii = TILE(Tall, i, i);
        double *yc = Ycopy + (size_t)i * t2, *tc = Tcopy + (size_t)i * t2;
        #pragma omp task depend(inout: aii[0]) depend(out: yc[0]) firstprivate(aii, tii, yc, tc, i)
        {
            orc_core_dgeqrt(NB, NB, IB, aii, NB, tii, NB, TAUP(TAU, i, i));
            memcpy(yc, aii, sizeof(double) * t2);
            memcpy(tc, tii, sizeof(double) * t2);
        }
        for (int j = i + 1; j < NT; j++) {
            double *aij = TILE(A, i, j);
            #pragma omp task depend(in: yc[0]) depend(inout: aij[0]) firstprivate(aij, yc, tc)
            orc_core_dormqr(NB, NB, NB, IB, yc, NB, tc, NB, aij, NB);
        }
        for (int k = i + 1; k < MT; k++) {
            double *aki = TILE(A, k, i), *tki = TILE(Tall, k, i);
            #pragma omp task depend(inout: aii[0], aki[0]) firstprivate(aii, aki, tki, k, i)
            orc_core_dtsqrt(NB, NB, IB, aii, NB, aki, NB, tki, NB, TAUP(TAU, k, i));
            for (int j = i + 1; j < NT; j++) {
                double *aij = TILE(A, i, j), *akj = TILE(A, k, j);
                #pragma omp task depend(in: aki[0]) depend(inout: aij[0], akj[0]) firstprivate(aij, akj, aki, tki)
                orc_core_dtsmqr(NB, NB, NB, NB, NB, IB, aij, NB, akj, NB, aki, NB, tki, NB);
            }
        }
    }
    free(Tall);
    free(Ycopy);
    free(Tcopy);
    return 0;
}

/* Hybrid_make_Q (Hybrid_make_Q.c:56-237) as a task DAG: the full-NB T of
 * every panel tile is built as a task, then each Q tile column runs its own
 * chain of LARFB/SSRFB tasks; V is zeroed at the end. */
ORC_EXPORT void orc_make_Q_dag(long M, long N, int NB, double *Q, double *RY, double *TAU)
{
    int MT = (int)(M / NB), NT = (int)(N / NB);
    int steps = imin(MT, NT);
    const size_t t2 = (size_t)NB * NB;
    double *Tall = (double *)calloc((size_t)M * (size_t)N, sizeof(double));
    double *Yd = (double *)calloc((size_t)steps * t2, sizeof(double));
    for (int c = 0; c < NT; c++) {
        double *q = TILE(Q, c, c);
        for (int r = 0; r < NB; r++) q[r + (long)r * NB] = 1.0;
    }
    #pragma omp parallel num_threads(orc_nthreads)
    #pragma omp single
    {
        for (int gi = 0; gi < steps; gi++) {
            double *ry = TILE(RY, gi, gi), *y = Yd + (size_t)gi * t2, *t = TILE(Tall, gi, gi);
            #pragma omp task depend(out: t[0]) firstprivate(ry, y, t, gi)
            {
                for (int ii = 0; ii < NB - 1; ii++) {
                    for (int r = ii + 1; r < NB; r++) y[r + (long)ii * NB] = ry[r + (long)ii * NB];
                    y[ii + (long)ii * NB] = 1.0;
                }
                y[t2 - 1] = 0.0;
                orc_dlarft_fc(NB, NB, y, NB, TAUP(TAU, gi, gi), t, NB);
            }
            for (int k = gi + 1; k < MT; k++) {
                double *v = TILE(RY, k, gi), *tk = TILE(Tall, k, gi);
                #pragma omp task depend(out: tk[0]) firstprivate(v, tk, k, gi)
                orc_dtsrft(NB, NB, NB, v, NB, TAUP(TAU, k, gi), tk, NB);
            }
        }
        for (int gi = 0; gi < steps; gi++) {
            double *y = Yd + (size_t)gi * t2, *t = TILE(Tall, gi, gi);
            for (int j = 0; j < NT; j++) {
                double *qij = TILE(Q, gi, j);
                #pragma omp task depend(in: t[0]) depend(inout: qij[0]) firstprivate(y, t, qij)
                orc_core_dormqr(NB, NB, NB, NB, y, NB, t, NB, qij, NB);
            }
            for (int k = gi + 1; k < MT; k++) {
                double *v = TILE(RY, k, gi), *tk = TILE(Tall, k, gi);
                for (int j = 0; j < NT; j++) {
                    double *qij = TILE(Q, gi, j), *qkj = TILE(Q, k, j);
                    #pragma omp task depend(in: tk[0]) depend(inout: qij[0], qkj[0]) firstprivate(v, tk, qij, qkj)
                    orc_core_dtsmqr(NB, NB, NB, NB, NB, NB, qij, NB, qkj, NB, v, NB, tk, NB);
                }
            }
        }
    }
    for (int gi = 0; gi < steps; gi++) {
        double *ry = TILE(RY, gi, gi);
        for (int c = 0; c < NB; c++)
            for (int r = c + 1; r < NB; r++) ry[r + (long)c * NB] = 0.0;
        for (int k = gi + 1; k < MT; k++) memset(TILE(RY, k, gi), 0, sizeof(double) * t2);
    }
    free(Tall);
    free(Yd);
}
