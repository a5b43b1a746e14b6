/*
 * lapacke_shim.c -- LAPACKE_dsysv for column-major storage, restating
 * LAPACK's published algorithm: dsysv = dsytrf (for orders below the block
 * size, the unblocked Bunch-Kaufman factorisation dsytf2: A = U D U^T or
 * L D L^T with 1x1 and 2x2 pivot blocks, alpha = (1 + sqrt(17)) / 8) then
 * dsytrs.  The reference calls it on 3x3 systems with uplo 'U'
 * (DPRA/dpra_cpu.cpp:219).  TEST INFRASTRUCTURE ONLY
 * (oracle/ref_build.py); the element updates follow the reference BLAS
 * kernels' order (dsyr, dscal, dger, dgemv).
 */
#include <math.h>
#include <stddef.h>

#include "mkl.h"

#define A_(i, j) a[(i) + (size_t)(j) * lda] /* 0-based */

static int factor_upper(int n, double *a, int lda, int *ipiv)
{
    const double alpha = (1.0 + sqrt(17.0)) / 8.0;
    int info = 0;
    int k = n - 1;
    while (k >= 0) {
        int kstep = 1, kp;
        const double absakk = fabs(A_(k, k));
        int imax = 0;
        double colmax = 0.0;
        if (k > 0) {
            for (int i = 0; i < k; i++)
                if (fabs(A_(i, k)) > colmax) {
                    colmax = fabs(A_(i, k));
                    imax = i;
                }
        }
        if ((absakk > colmax ? absakk : colmax) == 0.0) {
            if (info == 0) info = k + 1;
            kp = k;
        } else {
            if (absakk >= alpha * colmax) {
                kp = k;
            } else {
                double rowmax = 0.0;
                for (int j = imax + 1; j <= k; j++)
                    if (fabs(A_(imax, j)) > rowmax) rowmax = fabs(A_(imax, j));
                if (imax > 0) {
                    double m = 0.0;
                    for (int i = 0; i < imax; i++)
                        if (fabs(A_(i, imax)) > m) m = fabs(A_(i, imax));
                    if (m > rowmax) rowmax = m;
                }
                if (absakk >= alpha * colmax * (colmax / rowmax)) {
                    kp = k;
                } else if (fabs(A_(imax, imax)) >= alpha * rowmax) {
                    kp = imax;
                } else {
                    kp = imax;
                    kstep = 2;
                }
            }
            const int kk = k - kstep + 1;
            if (kp != kk) {
                for (int i = 0; i < kp; i++) {
                    const double t = A_(i, kk);
                    A_(i, kk) = A_(i, kp);
                    A_(i, kp) = t;
                }
                for (int j = kp + 1; j < kk; j++) {
                    const double t = A_(j, kk);
                    A_(j, kk) = A_(kp, j);
                    A_(kp, j) = t;
                }
                double t = A_(kk, kk);
                A_(kk, kk) = A_(kp, kp);
                A_(kp, kp) = t;
                if (kstep == 2) {
                    t = A_(k - 1, k);
                    A_(k - 1, k) = A_(kp, k);
                    A_(kp, k) = t;
                }
            }
            if (kstep == 1) {
                /* A(0:k-1, 0:k-1) -= W W^T / D(k), W = A(0:k-1, k) (dsyr), then W /= D(k) (dscal) */
                const double r1 = 1.0 / A_(k, k);
                for (int j = 0; j < k; j++) {
                    const double temp = -r1 * A_(j, k);
                    for (int i = 0; i <= j; i++) A_(i, j) = A_(i, j) + A_(i, k) * temp;
                }
                for (int i = 0; i < k; i++) A_(i, k) = r1 * A_(i, k);
            } else if (k > 1) {
                double d12 = A_(k - 1, k);
                const double d22 = A_(k - 1, k - 1) / d12;
                const double d11 = A_(k, k) / d12;
                const double t = 1.0 / (d11 * d22 - 1.0);
                d12 = t / d12;
                for (int j = k - 2; j >= 0; j--) {
                    const double wkm1 = d12 * (d11 * A_(j, k - 1) - A_(j, k));
                    const double wk = d12 * (d22 * A_(j, k) - A_(j, k - 1));
                    for (int i = j; i >= 0; i--) A_(i, j) = A_(i, j) - A_(i, k) * wk - A_(i, k - 1) * wkm1;
                    A_(j, k) = wk;
                    A_(j, k - 1) = wkm1;
                }
            }
        }
        if (kstep == 1) {
            ipiv[k] = kp + 1;
        } else {
            ipiv[k] = -(kp + 1);
            ipiv[k - 1] = -(kp + 1);
        }
        k -= kstep;
    }
    return info;
}

static void solve_upper(int n, int nrhs, const double *a, int lda, const int *ipiv, double *b, int ldb)
{
#define B_(i, j) b[(i) + (size_t)(j) * ldb]
    /* U D X = B */
    int k = n - 1;
    while (k >= 0) {
        if (ipiv[k] > 0) {
            const int kp = ipiv[k] - 1;
            if (kp != k)
                for (int j = 0; j < nrhs; j++) {
                    const double t = B_(k, j);
                    B_(k, j) = B_(kp, j);
                    B_(kp, j) = t;
                }
            for (int j = 0; j < nrhs; j++) {
                const double temp = -B_(k, j);
                if (B_(k, j) != 0.0)
                    for (int i = 0; i < k; i++) B_(i, j) = B_(i, j) + A_(i, k) * temp;
            }
            const double r = 1.0 / A_(k, k);
            for (int j = 0; j < nrhs; j++) B_(k, j) = r * B_(k, j);
            k -= 1;
        } else {
            const int kp = -ipiv[k] - 1;
            if (kp != k - 1)
                for (int j = 0; j < nrhs; j++) {
                    const double t = B_(k - 1, j);
                    B_(k - 1, j) = B_(kp, j);
                    B_(kp, j) = t;
                }
            for (int j = 0; j < nrhs; j++) {
                double temp = -B_(k, j);
                if (B_(k, j) != 0.0)
                    for (int i = 0; i < k - 1; i++) B_(i, j) = B_(i, j) + A_(i, k) * temp;
                temp = -B_(k - 1, j);
                if (B_(k - 1, j) != 0.0)
                    for (int i = 0; i < k - 1; i++) B_(i, j) = B_(i, j) + A_(i, k - 1) * temp;
            }
            const double akm1k = A_(k - 1, k);
            const double akm1 = A_(k - 1, k - 1) / akm1k;
            const double ak = A_(k, k) / akm1k;
            const double denom = akm1 * ak - 1.0;
            for (int j = 0; j < nrhs; j++) {
                const double bkm1 = B_(k - 1, j) / akm1k;
                const double bk = B_(k, j) / akm1k;
                B_(k - 1, j) = (ak * bkm1 - bk) / denom;
                B_(k, j) = (akm1 * bk - bkm1) / denom;
            }
            k -= 2;
        }
    }
    /* U^T X = B */
    k = 0;
    while (k < n) {
        if (ipiv[k] > 0) {
            for (int j = 0; j < nrhs; j++) {
                double temp = 0.0;
                for (int i = 0; i < k; i++) temp = temp + A_(i, k) * B_(i, j);
                B_(k, j) = B_(k, j) - temp;
            }
            const int kp = ipiv[k] - 1;
            if (kp != k)
                for (int j = 0; j < nrhs; j++) {
                    const double t = B_(k, j);
                    B_(k, j) = B_(kp, j);
                    B_(kp, j) = t;
                }
            k += 1;
        } else {
            for (int j = 0; j < nrhs; j++) {
                double temp = 0.0;
                for (int i = 0; i < k; i++) temp = temp + A_(i, k) * B_(i, j);
                B_(k, j) = B_(k, j) - temp;
                temp = 0.0;
                for (int i = 0; i < k; i++) temp = temp + A_(i, k + 1) * B_(i, j);
                B_(k + 1, j) = B_(k + 1, j) - temp;
            }
            const int kp = -ipiv[k] - 1;
            if (kp != k)
                for (int j = 0; j < nrhs; j++) {
                    const double t = B_(k, j);
                    B_(k, j) = B_(kp, j);
                    B_(kp, j) = t;
                }
            k += 2;
        }
    }
#undef B_
}

lapack_int LAPACKE_dsysv(int matrix_layout, char uplo, lapack_int n, lapack_int nrhs, double *a, lapack_int lda,
                         lapack_int *ipiv, double *b, lapack_int ldb)
{
    if (matrix_layout != LAPACK_COL_MAJOR || (uplo != 'U' && uplo != 'u') || n < 0 || nrhs < 0 || lda < n ||
        ldb < n)
        return -1; /* only the form the reference calls */
    const int info = factor_upper(n, a, lda, ipiv);
    if (info > 0) return info;
    solve_upper(n, nrhs, a, lda, ipiv, b, ldb);
    return 0;
}
