/*
 * fftw_shim.c -- the FFTW3 subset declared in fftw3.h, on the oracle's
 * mixed-radix Stockham FFT.  TEST INFRASTRUCTURE ONLY (oracle/ref_build.py).
 * Each plan owns its scratch, so plans executed by different threads (the
 * reference keeps one per OpenMP thread, WFT/WFT2_CPU.cpp:741-760) are
 * independent.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

#define OR_REAL double
#define OR_FN(name) name##_d
#include "../or_fft_gen.h"

struct glsu_ref_fftw_plan {
    int n0, n1, inverse;
    double *in, *out;
    fft2_plan_d p;
};

void *fftw_malloc(size_t n) { return malloc(n ? n : 1); }
void fftw_free(void *p) { free(p); }
void *fftwf_malloc(size_t n) { return malloc(n ? n : 1); }
void fftwf_free(void *p) { free(p); }

fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign, unsigned flags)
{
    (void)flags;
    fftw_plan q = (fftw_plan)calloc(1, sizeof(*q));
    if (!q) return NULL;
    q->n0 = n0;
    q->n1 = n1;
    q->inverse = sign > 0;
    q->in = (double *)in;
    q->out = (double *)out;
    if (fft2_init_d(&q->p, n1, n0)) {
        free(q);
        return NULL;
    }
    return q;
}

void fftw_execute(const fftw_plan q)
{
    if (q->in != q->out) memcpy(q->out, q->in, sizeof(double) * 2 * (size_t)q->n0 * q->n1);
    fft2_exec_d(&((fftw_plan)q)->p, q->out, q->inverse);
}

void fftw_destroy_plan(fftw_plan q)
{
    if (!q) return;
    fft2_free_d(&q->p);
    free(q);
}
