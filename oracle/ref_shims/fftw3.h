/*
 * fftw3.h -- stand-in for the FFTW3 API subset that the reference's CPU WFF2
 * (WFT/WFT2_CPU.cpp, WFT/WFT.cpp, DPRA/dpra_cpu.cpp) calls, so that those
 * files compile here as they are.  TEST INFRASTRUCTURE ONLY: used by
 * oracle/ref_build.py to build oracle/_ref, which generates golden vectors.
 *
 * Semantics follow the FFTW3 manual: fftw_complex is double[2]; a 2-D plan
 * of n0 x n1 (row-major, n1 contiguous) computes the unnormalised DFT with
 * exponent sign `sign` (FFTW_FORWARD = -1, FFTW_BACKWARD = +1) from `in`
 * to `out` (in place when equal) at each fftw_execute.  The transforms are
 * the oracle's mixed-radix Stockham FFT (oracle/or_fft_gen.h), not FFTW.
 */
#ifndef GLSU_REF_FFTW3_SHIM_H
#define GLSU_REF_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef struct glsu_ref_fftw_plan *fftw_plan;
typedef struct glsu_ref_fftwf_plan *fftwf_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc(size_t n);
void fftw_free(void *p);
void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif

#endif
