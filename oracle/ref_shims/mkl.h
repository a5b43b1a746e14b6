/*
 * mkl.h -- stand-in for the one Intel MKL routine the reference's CPU DPRA
 * calls (LAPACKE_dsysv, DPRA/dpra_cpu.cpp:219), so that the file compiles
 * here as it is.  TEST INFRASTRUCTURE ONLY (oracle/ref_build.py).
 *
 * lapacke_shim.c restates LAPACK's published dsysv for a column-major
 * matrix: Bunch-Kaufman diagonal pivoting (dsytf2) and the matching solve
 * (dsytrs), unblocked, as LAPACK runs them for orders below its block size.
 */
#ifndef GLSU_REF_MKL_SHIM_H
#define GLSU_REF_MKL_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MKL_INT;
typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

lapack_int LAPACKE_dsysv(int matrix_layout, char uplo, lapack_int n, lapack_int nrhs, double *a, lapack_int lda,
                         lapack_int *ipiv, double *b, lapack_int ldb);

#ifdef __cplusplus
}
#endif

#endif
