/*
 * glsu_oracle_f32.c -- FP32 CPU restatement of the reference's float CPU
 * classes, for the timed CPU baseline.
 *
 * TEST INFRASTRUCTURE ONLY, like glsu_oracle.c: only the tests and the
 * CPU-baseline leg of the benchmark load it.  The parity oracle is the FP64
 * file; this one is the FP32 variant of the same frame, timed beside it.
 *
 * What is restated, and from where (paths inside the reference project):
 *   - DPRA_CPUF::dpra_per_frame, the per-pixel window sums in float and the
 *     3x3 solve (LAPACKE_ssysv; here Gaussian elimination with partial
 *     pivoting in float), dphi = atan2(-x3, x2):   DPRA/dpra_cpuf.cpp:130-230
 *   - the phase update in float:                    DPRA/dpra_cpuf.cpp:243-252
 *   - WFT2_cpuF::WFF2, the FFT formulation in float (fftwf here replaced by
 *     the oracle's Stockham FFT generated for float): WFT/WFT2_CPUf.cpp:190-390
 * As in the FP64 oracle: A00 = (2r+1)^2 for every window (the reference's
 * constant count), and the per-frequency-row partial sums are added in row
 * order after the sweep.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define OR_REAL float
#define OR_FN(name) name##_f
#include "or_fft_gen.h"
#undef OR_REAL
#undef OR_FN

int or_first_greater(int x);
int or_lut_value(int i);
int or_wff_count(double lo, double hi, double step);

/* Gaussian elimination with partial pivoting on a 3x3 float system; b -> x. */
static void solve3_gepp_f(float A[3][3], float b[3])
{
    for (int k = 0; k < 3; k++) {
        int piv = k;
        for (int i = k + 1; i < 3; i++)
            if (fabsf(A[i][k]) > fabsf(A[piv][k])) piv = i;
        if (piv != k) {
            for (int j = 0; j < 3; j++) { float t = A[k][j]; A[k][j] = A[piv][j]; A[piv][j] = t; }
            float t = b[k]; b[k] = b[piv]; b[piv] = t;
        }
        for (int i = k + 1; i < 3; i++) {
            float m = A[i][k] / A[k][k];
            for (int j = k; j < 3; j++) A[i][j] -= m * A[k][j];
            b[i] -= m * b[k];
        }
    }
    b[2] = b[2] / A[2][2];
    b[1] = (b[1] - A[1][2] * b[2]) / A[1][1];
    b[0] = (b[0] - A[0][1] * b[1] - A[0][2] * b[2]) / A[0][0];
}

/* DPRA least squares of one frame: z = exp(j dphi) per pixel (interleaved). */
void orf_dpra_ls(int W, int H, int r, const float *img, const float *phiref, float *z, int nthreads)
{
    const float a00 = (float)((2 * r + 1) * (2 * r + 1));
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < H; i++) {
        for (int j = 0; j < W; j++) {
            float sc = 0, ss = 0, scs = 0, ss2 = 0, sc2 = 0, sf = 0, sfc = 0, sfs = 0;
            int m0 = i - r < 0 ? 0 : i - r, m1 = i + r > H - 1 ? H - 1 : i + r;
            int n0 = j - r < 0 ? 0 : j - r, n1 = j + r > W - 1 ? W - 1 : j + r;
            for (int m = m0; m <= m1; m++)
                for (int n = n0; n <= n1; n++) {
                    size_t id = (size_t)m * W + n;
                    float c = cosf(phiref[id]), s = sinf(phiref[id]), ft = img[id];
                    sc += c; ss += s; scs += c * s; ss2 += s * s; sc2 += c * c;
                    sf += ft; sfc += ft * c; sfs += ft * s;
                }
            float A[3][3] = {{a00, sc, ss}, {sc, sc2, scs}, {ss, scs, ss2}};
            float b[3] = {sf, sfc, sfs};
            solve3_gepp_f(A, b);
            float d = atan2f(-b[2], b[1]);
            size_t id = (size_t)i * W + j;
            z[2 * id] = cosf(d);
            z[2 * id + 1] = sinf(d);
        }
    }
}

void orf_dpra_update(int N, const float *filtered, const float *phiref, const float *dphiref, float *phicurr,
                     float *dphi)
{
    for (int i = 0; i < N; i++) {
        float t = atan2f(filtered[2 * i + 1], filtered[2 * i]);
        phicurr[i] = atan2f(sinf(t + phiref[i]), cosf(t + phiref[i]));
        dphi[i] = dphiref[i] + t;
    }
}

/*
 * WFF2 in float, the FFT formulation of WFT2_cpuF::WFF2: per frequency the
 * windowed spectrum, sf = ifft2(Ff .* Fg), the hard threshold, the second
 * filter and the accumulation of the crop.  ky0, ky1: only frequency rows
 * y in [ky0, ky1) are swept (ky1 < 0: all), for bounded timing samples.
 * Returns 0, -1 when the padded size leaves the size table, -2 on no memory.
 */
int orf_wff2(int W, int H, const float *f, double sigx, double wxl, double wxh, double wxi, double sigy, double wyl,
             double wyh, double wyi, double thr_in, float *filtered, int nthreads, int ky0, int ky1)
{
    const int sx = (int)round(3 * sigx), sy = (int)round(3 * sigy);
    const int winW = 2 * sx + 1, winH = 2 * sy + 1;
    const int iH = or_first_greater(H + winH - 1), iW = or_first_greater(W + winW - 1);
    if (iH < 0 || iW < 0) return -1;
    const int Hp = or_lut_value(iH), Wp = or_lut_value(iW);
    const size_t P = (size_t)Hp * Wp;
    const size_t N = (size_t)H * W;

    float *g = (float *)calloc(2 * P, sizeof(float));
    float *Ff = (float *)calloc(2 * P, sizeof(float));
    if (!g || !Ff) {
        free(g);
        free(Ff);
        return -2;
    }
    float nrm = 0;
    for (int i = 0; i < winH; i++)
        for (int j = 0; j < winW; j++) {
            float y = (float)(i - (winH - 1) / 2), x = (float)(j - (winW - 1) / 2);
            float v = expf(-(x * x) / 2 / (float)sigx / (float)sigx - (y * y) / 2 / (float)sigy / (float)sigy);
            g[2 * ((size_t)i * Wp + j)] = v;
            nrm += v * v;
        }
    nrm = sqrtf(nrm);
    for (int i = 0; i < winH; i++)
        for (int j = 0; j < winW; j++) g[2 * ((size_t)i * Wp + j)] *= 1 / nrm;

    float thr = (float)thr_in;
    if (thr < 0) {
        float acc = 0;
        for (size_t k = 0; k < N; k++) acc += f[2 * k] * f[2 * k] + f[2 * k + 1] * f[2 * k + 1];
        thr = 6 * sqrtf(acc / (float)N / 3);
    }
    for (int i = 0; i < H; i++)
        for (int j = 0; j < W; j++) {
            Ff[2 * ((size_t)i * Wp + j)] = f[2 * ((size_t)i * W + j)];
            Ff[2 * ((size_t)i * Wp + j) + 1] = f[2 * ((size_t)i * W + j) + 1];
        }
    {
        fft2_plan_f p;
        if (fft2_init_f(&p, Wp, Hp)) return -2;
        fft2_exec_f(&p, Ff, 0);
        fft2_free_f(&p);
    }

    const int iwx = or_wff_count(wxl, wxh, wxi);
    const int iwy = or_wff_count(wyl, wyh, wyi);
    if (ky1 < 0 || ky1 > iwy) ky1 = iwy;
    if (ky0 < 0) ky0 = 0;
    const int nrows = ky1 > ky0 ? ky1 - ky0 : 0;
    float *part = (float *)calloc(2 * N * (size_t)(nrows ? nrows : 1), sizeof(float));
    if (!part) return -2;
    const float invP = 1.0f / (float)P;

#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        float *gw = (float *)malloc(sizeof(float) * 2 * P);
        float *Fg = (float *)malloc(sizeof(float) * 2 * P);
        float *Sf = (float *)malloc(sizeof(float) * 2 * P);
        fft2_plan_f p;
        fft2_init_f(&p, Wp, Hp);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int yy = ky0; yy < ky1; yy++) {
            float *acc = part + 2 * N * (size_t)(yy - ky0);
            for (int xx = 0; xx < iwx; xx++) {
                const float wyt = (float)(wyl + (double)yy * wyi);
                const float wxt = (float)(wxl + (double)xx * wxi);
                memset(gw, 0, sizeof(float) * 2 * P);
                for (int i = 0; i < winH; i++)
                    for (int j = 0; j < winW; j++) {
                        size_t id = (size_t)i * Wp + j;
                        float ys = (float)(i - (winH - 1) / 2), xs = (float)(j - (winW - 1) / 2);
                        float c = cosf(wxt * xs + wyt * ys), s = sinf(wxt * xs + wyt * ys);
                        gw[2 * id] = g[2 * id] * c;
                        gw[2 * id + 1] = g[2 * id] * s;
                    }
                memcpy(Fg, gw, sizeof(float) * 2 * P);
                fft2_exec_f(&p, Fg, 0);
                for (size_t k = 0; k < P; k++) {
                    float ar = Ff[2 * k], ai = Ff[2 * k + 1], br = Fg[2 * k], bi = Fg[2 * k + 1];
                    Sf[2 * k] = (ar * br - ai * bi) * invP;
                    Sf[2 * k + 1] = (ar * bi + ai * br) * invP;
                }
                fft2_exec_f(&p, Sf, 1);
                for (int i = 0; i < Hp; i++)
                    for (int j = 0; j < Wp; j++) {
                        size_t d = (size_t)i * Wp + j;
                        if (i < H && j < W) {
                            size_t s = (size_t)(i + sy) * Wp + (j + sx);
                            float re = Sf[2 * s], im = Sf[2 * s + 1];
                            int keep = sqrtf(re * re + im * im) >= thr;
                            gw[2 * d] = keep ? re : 0.0f;
                            gw[2 * d + 1] = keep ? im : 0.0f;
                        } else {
                            gw[2 * d] = 0;
                            gw[2 * d + 1] = 0;
                        }
                    }
                fft2_exec_f(&p, gw, 0);
                for (size_t k = 0; k < P; k++) {
                    float ar = gw[2 * k], ai = gw[2 * k + 1], br = Fg[2 * k], bi = Fg[2 * k + 1];
                    gw[2 * k] = (ar * br - ai * bi) * invP;
                    gw[2 * k + 1] = (ar * bi + ai * br) * invP;
                }
                fft2_exec_f(&p, gw, 1);
                for (int i = 0; i < H; i++)
                    for (int j = 0; j < W; j++) {
                        size_t s = (size_t)(i + sy) * Wp + (j + sx);
                        size_t d = (size_t)i * W + j;
                        acc[2 * d] += gw[2 * s];
                        acc[2 * d + 1] += gw[2 * s + 1];
                    }
            }
        }
        fft2_free_f(&p);
        free(gw);
        free(Fg);
        free(Sf);
    }

    const float scale = (float)(0.25 * (1.0 / (M_PI * M_PI)) * wxi * wyi);
    for (size_t k = 0; k < N; k++) {
        float re = 0, im = 0;
        for (int r = 0; r < nrows; r++) {
            re += part[2 * (N * (size_t)r + k)];
            im += part[2 * (N * (size_t)r + k) + 1];
        }
        filtered[2 * k] = re * scale;
        filtered[2 * k + 1] = im * scale;
    }
    free(part);
    free(g);
    free(Ff);
    return 0;
}
