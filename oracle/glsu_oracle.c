/*
 * glsu_oracle.c -- FP64 CPU restatement of the G-LS3U reference algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: only the tests,
 * the smoke check and the CPU-baseline leg of the benchmark may load it.  The
 * product (the CUDA library) never links, calls or falls back to it.
 *
 * What is restated, and from where (paths inside the reference project):
 *   - FFT size lookup table and its binary search:   WFT/WFT.h:18-32, WFT/WFT.cpp:10-23
 *   - WFF2 (windowed Fourier filtering), the CPU
 *     FFT formulation with the truncated window:      WFT/WFT2_CPU.cpp:190-390, 697-805, 815-845, 959-1022
 *   - DPRA per-pixel windowed least squares:          DPRA/dpra_cpu.cpp:130-230 (window radius r
 *     generalises the hard-wired 3x3; A00 = (2r+1)^2 keeps the reference's constant-count quirk)
 *   - DPRA phase update:                              DPRA/dpra_cpu.cpp:243-258
 *   - AIA alternating least squares:                  AIA/aia_cpu.cpp:16-263
 *   - ifftshift-ed integer frequency grid:            Test/xfyf_2D_1D_Test.cu:48-108 (golden Test/xfyf.csv)
 *   - line-scanning spatial unwrapping:               MatLab/fp_unwrapping.m:41-71
 *
 * Documented deviations (all FP64 throughout):
 *   - DPRA/dpra_cpu.cpp:246 truncates atan2 of the filtered value to float; here it stays double.
 *   - The DPRA normal equations are solved through the Schur complement
 *     with centre-shifted window sums (or_dpra_ls); the literal raw-sum form
 *     is kept as or_dpra_ls_raw.  See the comment above or_dpra_ls.
 *   - LAPACKE_dsysv (Bunch-Kaufman) is replaced by Gaussian elimination with
 *     partial pivoting and LAPACKE_dposv by a Cholesky solve; both give the
 *     same solution up to rounding for the matrices that arise.
 *   - FFTW/MKL is replaced by a self-written mixed-radix Stockham FFT.
 *   - WFF2 sums the per-frequency-row partial results in frequency order, so
 *     the result does not depend on the thread count (the reference sums
 *     per-thread partials, WFT/WFT2_CPU.cpp:358-372).
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

/* ------------------------------------------------------------------------ */
/* FFT size lookup table: even 2^a 3^b 5^c 7^d sizes up to 4096.            */
/* ------------------------------------------------------------------------ */
static int g_lut[512];
static int g_lut_n = 0;

static void lut_init(void)
{
    if (g_lut_n) return;
    int n = 0;
    for (int v = 2; v <= 4096; v += 2) {
        int t = v;
        while (t % 2 == 0) t /= 2;
        while (t % 3 == 0) t /= 3;
        while (t % 5 == 0) t /= 5;
        while (t % 7 == 0) t /= 7;
        if (t == 1) g_lut[n++] = v;
    }
    g_lut_n = n;
}

int or_fft_lut(int *out, int cap)
{
    lut_init();
    int n = g_lut_n < cap ? g_lut_n : cap;
    for (int i = 0; i < n; i++) out[i] = g_lut[i];
    return g_lut_n;
}

/* Index of the first LUT entry >= x, or -1 (WFT/WFT.cpp:10-23). */
/* Entry i of the size table (used by the FP32 variant, glsu_oracle_f32.c). */
int or_lut_value(int i)
{
    lut_init();
    return g_lut[i];
}

int or_first_greater(int x)
{
    lut_init();
    int first = 0, last = g_lut_n - 1;
    while (first <= last) {
        int mid = (first + last) / 2;
        if (g_lut[mid] >= x) last = mid - 1;
        else first = mid + 1;
    }
    return (last + 1 == g_lut_n) ? -1 : last + 1;
}

int or_opt_fft_size(int x)
{
    int i = or_first_greater(x);
    return i < 0 ? -1 : g_lut[i];
}

/* ifftshift-ed integer frequency grid of a W x H plane. */
void or_freq_grid(int W, int H, double *xf, double *yf)
{
    for (int i = 0; i < H; i++)
        for (int j = 0; j < W; j++) {
            xf[i * W + j] = (double)(((j + W / 2) % W) - W / 2);
            yf[i * W + j] = (double)(((i + H / 2) % H) - H / 2);
        }
}

#define OR_REAL double
#define OR_FN(name) name
#include "or_fft_gen.h"
#undef OR_REAL
#undef OR_FN

/* Exposed for the oracle's own self-test against numpy.fft. */
int or_fft1d(int n, double *x, int inverse)
{
    fft_plan p;
    if (fft_plan_init(&p, n)) return -1;
    double *s = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    fft_exec(&p, x, s, inverse);
    free(s);
    fft_plan_free(&p);
    return 0;
}

int or_fft2d(int W, int H, double *x, int inverse)
{
    fft2_plan p;
    if (fft2_init(&p, W, H)) return -1;
    fft2_exec(&p, x, inverse);
    fft2_free(&p);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* WFF2 -- WFT/WFT2_CPU.cpp:190-390 (+ initialisation 697-845, 959-1022).   */
/* ------------------------------------------------------------------------ */
int or_wff_count(double lo, double hi, double step)
{
    /* WFT/WFT2_CPU.cpp:222-223 */
    return (int)((hi - lo) * (1.0 / step)) + 1;
}

/*
 * f:        H*W complex (interleaved) input.
 * filtered: H*W complex output.
 * thr:      threshold; thr < 0 selects 6*sqrt(mean(|f|^2)/3) (WFT2_CPU.cpp:977-1005).
 * ky0, ky1: only frequency rows y in [ky0, ky1) are swept (ky1 < 0: all).
 *           Used for bounded CPU-baseline samples; tests use the full sweep.
 * Returns 0, or -1 when the padded size leaves the LUT (the reference throws -1).
 */
int or_wff2(int W, int H, const double *f, double sigx, double wxl, double wxh, double wxi,
            double sigy, double wyl, double wyh, double wyi, double thr, double *filtered,
            double *thr_used, int nthreads, int ky0, int ky1)
{
    const int sx = (int)round(3 * sigx), sy = (int)round(3 * sigy);
    const int winW = 2 * sx + 1, winH = 2 * sy + 1;
    const int iH = or_first_greater(H + winH - 1), iW = or_first_greater(W + winW - 1);
    if (iH < 0 || iW < 0) return -1;
    const int Hp = g_lut[iH], Wp = g_lut[iW];
    const size_t P = (size_t)Hp * Wp;
    const size_t N = (size_t)H * W;

    /* window g, normalised by its L2 norm (WFT2_CPU.cpp:766-807) */
    double *g = (double *)calloc(2 * P, sizeof(double));
    double *Ff = (double *)calloc(2 * P, sizeof(double));
    if (!g || !Ff) return -2;
    double nrm = 0;
    for (int i = 0; i < winH; i++)
        for (int j = 0; j < winW; j++) {
            double y = (double)(i - (winH - 1) / 2), x = (double)(j - (winW - 1) / 2);
            double v = exp(-(x * x) / 2 / sigx / sigx - (y * y) / 2 / sigy / sigy);
            g[2 * ((size_t)i * Wp + j)] = v;
            nrm += v * v;
        }
    nrm = sqrt(nrm);
    for (int i = 0; i < winH; i++)
        for (int j = 0; j < winW; j++) g[2 * ((size_t)i * Wp + j)] *= 1 / nrm;

    /* threshold + feed (WFT2_CPU.cpp:977-1022) */
    if (thr < 0) {
        double acc = 0;
        for (size_t k = 0; k < N; k++) {
            double a = sqrt(f[2 * k] * f[2 * k] + f[2 * k + 1] * f[2 * k + 1]);
            acc += a * a;
        }
        acc = acc / (double)N / 3;
        thr = 6 * sqrt(acc);
    }
    if (thr_used) *thr_used = thr;
    for (int i = 0; i < H; i++)
        for (int j = 0; j < W; j++) {
            Ff[2 * ((size_t)i * Wp + j)] = f[2 * ((size_t)i * W + j)];
            Ff[2 * ((size_t)i * Wp + j) + 1] = f[2 * ((size_t)i * W + j) + 1];
        }
    {
        fft2_plan p;
        if (fft2_init(&p, Wp, Hp)) return -2;
        fft2_exec(&p, Ff, 0);
        fft2_free(&p);
    }

    const int iwx = or_wff_count(wxl, wxh, wxi);
    const int iwy = or_wff_count(wyl, wyh, wyi);
    if (ky1 < 0 || ky1 > iwy) ky1 = iwy;
    if (ky0 < 0) ky0 = 0;
    const int nrows = ky1 > ky0 ? ky1 - ky0 : 0;
    double *part = (double *)calloc(2 * N * (size_t)(nrows ? nrows : 1), sizeof(double));
    if (!part) return -2;
    const double invP = 1.0 / (double)P;

#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        double *gw = (double *)malloc(sizeof(double) * 2 * P);
        double *Fg = (double *)malloc(sizeof(double) * 2 * P);
        double *Sf = (double *)malloc(sizeof(double) * 2 * P);
        fft2_plan p;
        fft2_init(&p, Wp, Hp);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int yy = ky0; yy < ky1; yy++) {
            double *acc = part + 2 * N * (size_t)(yy - ky0);
            for (int xx = 0; xx < iwx; xx++) {
                const double wyt = wyl + (double)yy * wyi;
                const double wxt = wxl + (double)xx * wxi;
                /* gwave = g .* exp(j(wxt x + wyt y)) (WFT2_CPU.cpp:247-266) */
                memset(gw, 0, sizeof(double) * 2 * P);
                for (int i = 0; i < winH; i++)
                    for (int j = 0; j < winW; j++) {
                        size_t id = (size_t)i * Wp + j;
                        double ys = (double)(i - (winH - 1) / 2), xs = (double)(j - (winW - 1) / 2);
                        double c = cos(wxt * xs + wyt * ys), s = sin(wxt * xs + wyt * ys);
                        gw[2 * id] = g[2 * id] * c;
                        gw[2 * id + 1] = g[2 * id] * s;
                    }
                memcpy(Fg, gw, sizeof(double) * 2 * P);
                fft2_exec(&p, Fg, 0);
                /* sf = ifft2(Ff .* Fg) (WFT2_CPU.cpp:270-285) */
                for (size_t k = 0; k < P; k++) {
                    double ar = Ff[2 * k], ai = Ff[2 * k + 1], br = Fg[2 * k], bi = Fg[2 * k + 1];
                    Sf[2 * k] = (ar * br - ai * bi) * invP;
                    Sf[2 * k + 1] = (ar * bi + ai * br) * invP;
                }
                fft2_exec(&p, Sf, 1);
                /* crop at (sy, sx) and hard-threshold |sf| >= thr into the
                 * top-left H x W block, zero elsewhere (net effect of the
                 * in-place loop at WFT2_CPU.cpp:287-319). */
                for (int i = 0; i < Hp; i++)
                    for (int j = 0; j < Wp; j++) {
                        size_t d = (size_t)i * Wp + j;
                        if (i < H && j < W) {
                            size_t s = (size_t)(i + sy) * Wp + (j + sx);
                            double re = Sf[2 * s], im = Sf[2 * s + 1];
                            double a = sqrt(re * re + im * im);
                            gw[2 * d] = (a >= thr) ? re : 0.0;
                            gw[2 * d + 1] = (a >= thr) ? im : 0.0;
                        } else {
                            gw[2 * d] = 0;
                            gw[2 * d + 1] = 0;
                        }
                    }
                /* ifft2(fft2(sf) .* Fg) (WFT2_CPU.cpp:321-339) */
                fft2_exec(&p, gw, 0);
                for (size_t k = 0; k < P; k++) {
                    double ar = gw[2 * k], ai = gw[2 * k + 1], br = Fg[2 * k], bi = Fg[2 * k + 1];
                    gw[2 * k] = (ar * br - ai * bi) * invP;
                    gw[2 * k + 1] = (ar * bi + ai * br) * invP;
                }
                fft2_exec(&p, gw, 1);
                /* accumulate the crop (WFT2_CPU.cpp:341-352) */
                for (int i = 0; i < H; i++)
                    for (int j = 0; j < W; j++) {
                        size_t s = (size_t)(i + sy) * Wp + (j + sx);
                        size_t d = (size_t)i * W + j;
                        acc[2 * d] += gw[2 * s];
                        acc[2 * d + 1] += gw[2 * s + 1];
                    }
            }
        }
        fft2_free(&p);
        free(gw);
        free(Fg);
        free(Sf);
    }

    /* sum in frequency-row order, then scale by wxi*wyi/(4 pi^2) (WFT2_CPU.cpp:375-389) */
    const double scale = 0.25 * (1.0 / (M_PI * M_PI)) * wxi * wyi;
    for (size_t k = 0; k < N; k++) {
        double re = 0, im = 0;
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

/*
 * WFR2, windowed Fourier ridges (WFT/WFT2_CPU.cpp:391-694, WFR2_Init
 * :846-956): for every frequency of the grid, sf = f conv (g e^{j(wx x + wy y)})
 * by FFT as in or_wff2; per pixel the largest |sf| (ties: the later
 * frequency in wy-major, wx-minor order, as the single-thread loop with
 * `>=` at :505-518), its wx, wy and angle; then the curvature least squares
 * cxx = -conv2(wx, x.*g, 'same') / sum(x.*x.*g) with the map replicated
 * beyond the border (:551-631, :636-671), cyy alike, the compensated phase
 * and the amplitude (:674-692).
 * out: 8 arrays of H*W doubles: wx, wy, phase, phase_comp, b, r, cxx, cyy.
 * Returns 0, or -1 when the padded size leaves the LUT.
 */
int or_wfr2(int W, int H, const double *f, double sigx, double wxl, double wxh, double wxi, double sigy,
            double wyl, double wyh, double wyi, double *wx, double *wy, double *phase, double *phase_comp,
            double *b, double *r, double *cxx, double *cyy, int nthreads)
{
    const int sx = (int)round(3 * sigx), sy = (int)round(3 * sigy);
    const int winW = 2 * sx + 1, winH = 2 * sy + 1;
    const int iH = or_first_greater(H + winH - 1), iW = or_first_greater(W + winW - 1);
    if (iH < 0 || iW < 0) return -1;
    const int Hp = g_lut[iH], Wp = g_lut[iW];
    const size_t P = (size_t)Hp * Wp;
    const size_t N = (size_t)H * W;

    double *g = (double *)calloc((size_t)winH * winW, sizeof(double));
    double *Ff = (double *)calloc(2 * P, sizeof(double));
    if (!g || !Ff) return -2;
    double nrm = 0;
    for (int i = 0; i < winH; i++)
        for (int j = 0; j < winW; j++) {
            double y = (double)(i - (winH - 1) / 2), x = (double)(j - (winW - 1) / 2);
            double v = exp(-(x * x) / 2 / sigx / sigx - (y * y) / 2 / sigy / sigy);
            g[(size_t)i * winW + j] = v;
            nrm += v * v;
        }
    nrm = sqrt(nrm);
    for (size_t k = 0; k < (size_t)winH * winW; k++) g[k] *= 1 / nrm;
    for (int i = 0; i < H; i++)
        for (int j = 0; j < W; j++) {
            Ff[2 * ((size_t)i * Wp + j)] = f[2 * ((size_t)i * W + j)];
            Ff[2 * ((size_t)i * Wp + j) + 1] = f[2 * ((size_t)i * W + j) + 1];
        }
    {
        fft2_plan p;
        if (fft2_init(&p, Wp, Hp)) return -2;
        fft2_exec(&p, Ff, 0);
        fft2_free(&p);
    }
    const int iwx = or_wff_count(wxl, wxh, wxi), iwy = or_wff_count(wyl, wyh, wyi);
    /* per frequency row: best |sf|, its wx index and angle (ties: later wx) */
    double *pr = (double *)malloc(sizeof(double) * N * (size_t)iwy);
    double *pp = (double *)malloc(sizeof(double) * N * (size_t)iwy);
    int *px = (int *)malloc(sizeof(int) * N * (size_t)iwy);
    if (!pr || !pp || !px) return -2;
    const double invP = 1.0 / (double)P;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        double *Fg = (double *)malloc(sizeof(double) * 2 * P);
        double *Sf = (double *)malloc(sizeof(double) * 2 * P);
        fft2_plan p;
        fft2_init(&p, Wp, Hp);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int yy = 0; yy < iwy; yy++) {
            double *rr = pr + N * (size_t)yy, *ph = pp + N * (size_t)yy;
            int *ix = px + N * (size_t)yy;
            for (size_t k = 0; k < N; k++) {
                rr[k] = 0;
                ph[k] = 0;
                ix[k] = 0;
            }
            for (int xx = 0; xx < iwx; xx++) {
                const double wyt = wyl + (double)yy * wyi, wxt = wxl + (double)xx * wxi;
                memset(Fg, 0, sizeof(double) * 2 * P);
                for (int i = 0; i < winH; i++)
                    for (int j = 0; j < winW; j++) {
                        size_t id = (size_t)i * Wp + j;
                        double ys = (double)(i - (winH - 1) / 2), xs = (double)(j - (winW - 1) / 2);
                        double gv = g[(size_t)i * winW + j];
                        Fg[2 * id] = gv * cos(wxt * xs + wyt * ys);
                        Fg[2 * id + 1] = gv * sin(wxt * xs + wyt * ys);
                    }
                fft2_exec(&p, Fg, 0);
                for (size_t k = 0; k < P; k++) {
                    double ar = Ff[2 * k], ai = Ff[2 * k + 1], br = Fg[2 * k], bi = Fg[2 * k + 1];
                    Sf[2 * k] = (ar * br - ai * bi) * invP;
                    Sf[2 * k + 1] = (ar * bi + ai * br) * invP;
                }
                fft2_exec(&p, Sf, 1);
                for (int i = 0; i < H; i++)
                    for (int j = 0; j < W; j++) {
                        size_t s = (size_t)(i + sy) * Wp + (j + sx), d = (size_t)i * W + j;
                        double re = Sf[2 * s], im = Sf[2 * s + 1];
                        double a = sqrt(re * re + im * im);
                        if (a >= rr[d]) {
                            rr[d] = a;
                            ix[d] = xx;
                            ph[d] = atan2(im, re);
                        }
                    }
            }
        }
        fft2_free(&p);
        free(Fg);
        free(Sf);
    }
    /* merge the frequency rows in order with `>=` */
    for (size_t k = 0; k < N; k++) {
        double best = 0, ph = 0;
        int bx = 0, by = 0;
        for (int yy = 0; yy < iwy; yy++) {
            double a = pr[N * (size_t)yy + k];
            if (a >= best) {
                best = a;
                bx = px[N * (size_t)yy + k];
                by = yy;
                ph = pp[N * (size_t)yy + k];
            }
        }
        r[k] = best;
        wx[k] = wxl + (double)bx * wxi;
        wy[k] = wyl + (double)by * wyi;
        phase[k] = ph;
    }
    free(pr);
    free(pp);
    free(px);

    /* curvature least squares with the border pixel replicated */
    double sxx = 0, syy = 0;
    for (int i = 0; i < winH; i++)
        for (int j = 0; j < winW; j++) {
            double y = (double)(i - sy), x = (double)(j - sx);
            sxx += x * x * g[(size_t)i * winW + j];
            syy += y * y * g[(size_t)i * winW + j];
        }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < H; i++)
        for (int j = 0; j < W; j++) {
            double ax = 0, ay = 0;
            for (int a = 0; a < winH; a++) {
                const int m = a - sy;
                int yi = i - m;
                yi = yi < 0 ? 0 : (yi > H - 1 ? H - 1 : yi);
                for (int c = 0; c < winW; c++) {
                    const int n = c - sx;
                    int xi = j - n;
                    xi = xi < 0 ? 0 : (xi > W - 1 ? W - 1 : xi);
                    const double gv = g[(size_t)a * winW + c];
                    ax += gv * (double)n * wx[(size_t)yi * W + xi];
                    ay += gv * (double)m * wy[(size_t)yi * W + xi];
                }
            }
            const size_t k = (size_t)i * W + j;
            cxx[k] = -ax / sxx;
            cyy[k] = -ay / syy;
            double pc = phase[k] - 0.5 * atan(sigx * sigx * cxx[k]) - 0.5 * atan(sigy * sigy * cyy[k]);
            phase_comp[k] = atan2(sin(pc), cos(pc));
            b[k] = r[k] * pow((1 + sigx * sigx * sigx * sigx * cxx[k] * cxx[k]) * 0.25 / M_PI / (sigx * sigx), 0.25) *
                   pow((1 + sigy * sigy * sigy * sigy * cyy[k] * cyy[k]) * 0.25 / M_PI / (sigy * sigy), 0.25);
        }
    free(g);
    free(Ff);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Small dense solves.                                                      */
/* ------------------------------------------------------------------------ */
/* Gaussian elimination with partial pivoting on a 3x3 system; b -> x. */
static void solve3_gepp(double A[3][3], double b[3])
{
    for (int k = 0; k < 3; k++) {
        int piv = k;
        for (int i = k + 1; i < 3; i++)
            if (fabs(A[i][k]) > fabs(A[piv][k])) piv = i;
        if (piv != k) {
            for (int j = 0; j < 3; j++) { double t = A[k][j]; A[k][j] = A[piv][j]; A[piv][j] = t; }
            double t = b[k]; b[k] = b[piv]; b[piv] = t;
        }
        for (int i = k + 1; i < 3; i++) {
            double m = A[i][k] / A[k][k];
            for (int j = k; j < 3; j++) A[i][j] -= m * A[k][j];
            b[i] -= m * b[k];
        }
    }
    b[2] = b[2] / A[2][2];
    b[1] = (b[1] - A[1][2] * b[2]) / A[1][1];
    b[0] = (b[0] - A[0][1] * b[1] - A[0][2] * b[2]) / A[0][0];
}

/* Cholesky A = U^T U of an SPD 3x3 matrix, then solve for nrhs columns. */
static int chol3_solve(const double A[3][3], double *B, int nrhs)
{
    double U[3][3] = {{0}};
    for (int j = 0; j < 3; j++) {
        double s = A[j][j];
        for (int k = 0; k < j; k++) s -= U[k][j] * U[k][j];
        if (s <= 0) return j + 1;
        U[j][j] = sqrt(s);
        for (int i = j + 1; i < 3; i++) {
            double t = A[j][i];
            for (int k = 0; k < j; k++) t -= U[k][j] * U[k][i];
            U[j][i] = t / U[j][j];
        }
    }
    for (int c = 0; c < nrhs; c++) {
        double *b = B + 3 * (size_t)c;
        double y[3];
        for (int i = 0; i < 3; i++) {
            double t = b[i];
            for (int k = 0; k < i; k++) t -= U[k][i] * y[k];
            y[i] = t / U[i][i];
        }
        for (int i = 2; i >= 0; i--) {
            double t = y[i];
            for (int k = i + 1; k < 3; k++) t -= U[i][k] * b[k];
            b[i] = t / U[i][i];
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* DPRA -- DPRA/dpra_cpu.cpp:130-230 with window radius r.                  */
/* ------------------------------------------------------------------------ */
/*
 * img:    H*W intensities (double).
 * phiref: H*W reference phase.
 * z:      H*W complex output exp(j dphi).
 *
 * or_dpra_ls_raw follows DPRA/dpra_cpu.cpp:169-229 literally: raw window
 * sums, the 3x3 system with A00 = (2r+1)^2, a pivoted solve.
 *
 * or_dpra_ls solves the same normal equations in a numerically stable way:
 * x1 is eliminated (Schur complement) and the 2x2 system for (x2, x3) is
 * built from window sums of c, s, I shifted by the centre pixel's values.
 * In exact arithmetic both give the same dphi.  Where phi_ref is locally
 * smooth the 3x3 raw-sum matrix has a condition number of 1e6-1e10 and the
 * literal form loses that many digits (up to ~1e-3 rad at FP64 on the
 * benchmark sequences); the shifted form does not, so it is the parity
 * reference for the FP64 bar.  With rho = 1 - cnt/n0 (cnt = pixels inside
 * the clipped window, n0 = (2r+1)^2) and P* the shifted sums:
 *   a = Pcc - Pc^2/n0 + rho (2 mc Pc + cnt mc^2)      (and d, b, p, q alike)
 *   x2 ~ d p - b q,  x3 ~ a q - b p,  dphi = atan2(-x3, x2)
 */
void or_dpra_ls_raw(int W, int H, int r, const double *img, const double *phiref, double *z, int nthreads)
{
    const double a00 = (double)((2 * r + 1) * (2 * r + 1));
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < H; i++) {
        for (int j = 0; j < W; j++) {
            double sc = 0, ss = 0, scs = 0, ss2 = 0, sc2 = 0, sf = 0, sfc = 0, sfs = 0;
            int m0 = i - r < 0 ? 0 : i - r, m1 = i + r > H - 1 ? H - 1 : i + r;
            int n0 = j - r < 0 ? 0 : j - r, n1 = j + r > W - 1 ? W - 1 : j + r;
            for (int m = m0; m <= m1; m++)
                for (int n = n0; n <= n1; n++) {
                    size_t id = (size_t)m * W + n;
                    double c = cos(phiref[id]), s = sin(phiref[id]), ft = img[id];
                    sc += c; ss += s; scs += c * s; ss2 += s * s; sc2 += c * c;
                    sf += ft; sfc += ft * c; sfs += ft * s;
                }
            double A[3][3] = {{a00, sc, ss}, {sc, sc2, scs}, {ss, scs, ss2}};
            double b[3] = {sf, sfc, sfs};
            solve3_gepp(A, b);
            double d = atan2(-b[2], b[1]);
            size_t id = (size_t)i * W + j;
            z[2 * id] = cos(d);
            z[2 * id + 1] = sin(d);
        }
    }
}

void or_dpra_ls(int W, int H, int r, const double *img, const double *phiref, double *z, int nthreads)
{
    const double n0 = (double)((2 * r + 1) * (2 * r + 1));
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < H; i++) {
        for (int j = 0; j < W; j++) {
            const size_t id = (size_t)i * W + j;
            const double mc = cos(phiref[id]), ms = sin(phiref[id]), mi = img[id];
            double pc = 0, ps = 0, pi = 0, pcc = 0, pss = 0, pcs = 0, pic = 0, pis = 0;
            int m0 = i - r < 0 ? 0 : i - r, m1 = i + r > H - 1 ? H - 1 : i + r;
            int n0i = j - r < 0 ? 0 : j - r, n1 = j + r > W - 1 ? W - 1 : j + r;
            for (int m = m0; m <= m1; m++)
                for (int n = n0i; n <= n1; n++) {
                    size_t q = (size_t)m * W + n;
                    double dc = cos(phiref[q]) - mc, ds = sin(phiref[q]) - ms, di = img[q] - mi;
                    pc += dc; ps += ds; pi += di;
                    pcc += dc * dc; pss += ds * ds; pcs += dc * ds; pic += di * dc; pis += di * ds;
                }
            const double cnt = (double)((m1 - m0 + 1) * (n1 - n0i + 1));
            const double rho = 1.0 - cnt / n0;
            const double a = pcc - pc * pc / n0 + rho * (2 * mc * pc + cnt * mc * mc);
            const double d = pss - ps * ps / n0 + rho * (2 * ms * ps + cnt * ms * ms);
            const double b = pcs - pc * ps / n0 + rho * (mc * ps + ms * pc + cnt * mc * ms);
            const double p = pic - pi * pc / n0 + rho * (mi * pc + mc * pi + cnt * mi * mc);
            const double q = pis - pi * ps / n0 + rho * (mi * ps + ms * pi + cnt * mi * ms);
            double X = d * p - b * q, Y = a * q - b * p;
            if (a * d - b * b < 0) { X = -X; Y = -Y; }
            const double h = hypot(X, Y);
            z[2 * id] = h > 0 ? X / h : 1.0;
            z[2 * id + 1] = h > 0 ? -Y / h : 0.0;
        }
    }
}

/* DPRA/dpra_cpu.cpp:243-249 (FP64 throughout). */
void or_dpra_update(int N, const double *filtered, const double *phiref, const double *dphiref,
                    double *phicurr, double *dphi)
{
    for (int i = 0; i < N; i++) {
        double t = atan2(filtered[2 * i + 1], filtered[2 * i]);
        phicurr[i] = atan2(sin(t + phiref[i]), cos(t + phiref[i]));
        dphi[i] = dphiref[i] + t;
    }
}

/* ------------------------------------------------------------------------ */
/* AIA -- AIA/aia_cpu.cpp:16-263.                                           */
/* ------------------------------------------------------------------------ */
/* computePhi (aia_cpu.cpp:102-170); x (N*3) receives the per-pixel solutions. */
static int aia_compute_phi(int M, int N, const double *f, const double *delta, double *phi, double *x)
{
    double a3 = 0, a4 = 0, a6 = 0, a7 = 0, a8 = 0;
    for (int i = 0; i < M; i++) {
        double c = cos(delta[i]), s = sin(delta[i]);
        a3 += c; a4 += c * c; a6 += s; a7 += c * s; a8 += s * s;
    }
    double A[3][3] = {{(double)M, a3, a6}, {a3, a4, a7}, {a6, a7, a8}};
    double *cd = (double *)malloc(sizeof(double) * 2 * (size_t)M);
    for (int i = 0; i < M; i++) { cd[2 * i] = cos(delta[i]); cd[2 * i + 1] = sin(delta[i]); }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int j = 0; j < N; j++) {
        double b0 = 0, b1 = 0, b2 = 0;
        for (int i = 0; i < M; i++) {
            double I = f[(size_t)i * N + j];
            b0 += I; b1 += I * cd[2 * i]; b2 += I * cd[2 * i + 1];
        }
        x[3 * (size_t)j] = b0; x[3 * (size_t)j + 1] = b1; x[3 * (size_t)j + 2] = b2;
    }
    free(cd);
    int info = chol3_solve(A, x, N);
    if (info) return info;
    for (int j = 0; j < N; j++) phi[j] = atan2(-x[3 * (size_t)j + 2], x[3 * (size_t)j + 1]);
    return 0;
}

/* computeDelta (aia_cpu.cpp:172-247). */
static int aia_compute_delta(int M, int N, const double *f, const double *phi, double *delta)
{
    double a3 = 0, a4 = 0, a6 = 0, a7 = 0, a8 = 0;
    for (int j = 0; j < N; j++) {
        double c = cos(phi[j]), s = sin(phi[j]);
        a3 += c; a4 += c * c; a6 += s; a7 += c * s; a8 += s * s;
    }
    double A[3][3] = {{(double)N, a3, a6}, {a3, a4, a7}, {a6, a7, a8}};
    double *B = (double *)calloc(3 * (size_t)M, sizeof(double));
    for (int i = 0; i < M; i++) {
        double b0 = 0, b1 = 0, b2 = 0;
        for (int j = 0; j < N; j++) {
            double I = f[(size_t)i * N + j];
            b0 += I; b1 += I * cos(phi[j]); b2 += I * sin(phi[j]);
        }
        B[3 * i] = b0; B[3 * i + 1] = b1; B[3 * i + 2] = b2;
    }
    int info = chol3_solve(A, B, M);
    if (!info)
        for (int i = 0; i < M; i++) delta[i] = atan2(-B[3 * i + 2], B[3 * i + 1]);
    free(B);
    return info;
}

/* One per-pixel solve with given deltas: the quantity Test/Phi_CPU.csv pins. */
int or_aia_phi_solve(int M, int N, const double *f, const double *delta, double *phi, double *x)
{
    return aia_compute_phi(M, N, f, delta, phi, x);
}

/*
 * Full AIA (aia_cpu.cpp:16-100).  delta (M) holds the initial deltas on entry
 * and the normalised deltas on exit; phi (N) receives the wrapped phase.
 * rel = 0: the convergence measure of aia_cpu.cpp:249-263, max |delta - old|;
 * rel = 1: that of AIA_CUDAF_YC2 (aia_cudaf_v2.cu:665-677), the change of
 * delta_i - delta_0.
 */
int or_aia_mode(int M, int N, const double *f, double *delta, int max_iter, double max_err, int rel, double *phi,
                int *iters, double *err)
{
    double *x = (double *)malloc(sizeof(double) * 3 * (size_t)N);
    double *old = (double *)malloc(sizeof(double) * (size_t)M);
    double e = max_err * 2.0;
    int it = 0, info = 0;
    while (e > max_err && it < max_iter) {
        memcpy(old, delta, sizeof(double) * M);
        if ((info = aia_compute_phi(M, N, f, delta, phi, x))) break;
        if ((info = aia_compute_delta(M, N, f, phi, delta))) break;
        it++;
        e = 0;
        for (int i = 0; i < M; i++) {
            double d = rel ? fabs((delta[i] - delta[0]) - (old[i] - old[0])) : fabs(delta[i] - old[i]);
            if (d > e) e = d;
        }
    }
    if (!info) info = aia_compute_phi(M, N, f, delta, phi, x);
    if (!info) {
        for (int j = 0; j < N; j++) {
            phi[j] += delta[0];
            phi[j] = atan2(sin(phi[j]), cos(phi[j]));
        }
        for (int i = M - 1; i >= 0; i--) {
            delta[i] -= delta[0];
            delta[i] = atan2(sin(delta[i]), cos(delta[i]));
        }
    }
    *iters = it;
    *err = e;
    free(x);
    free(old);
    return info;
}

int or_aia(int M, int N, const double *f, double *delta, int max_iter, double max_err, double *phi,
           int *iters, double *err)
{
    return or_aia_mode(M, N, f, delta, max_iter, max_err, 0, phi, iters, err);
}

/* ------------------------------------------------------------------------ */
/* Line-scanning spatial unwrapping -- MatLab/fp_unwrapping.m:41-71 (the    */
/* MATLAB spec; the C++ reference omits it).  p: H*W row-major, in place;   */
/* start_row/start_col are 0-based.  round() is MATLAB's (half away from 0). */
/* ------------------------------------------------------------------------ */
static void unwrap1(double *p, int n, size_t stride, int s)
{
    const double tp = 2.0 * M_PI;
    for (int i = s + 1; i < n; i++)
        p[i * stride] += round((p[(i - 1) * stride] - p[i * stride]) / tp) * tp;
    for (int i = s - 1; i >= 0; i--)
        p[i * stride] += round((p[(i + 1) * stride] - p[i * stride]) / tp) * tp;
}

void or_unwrap2(int W, int H, double *p, int start_row, int start_col)
{
    /* seed column, from start_row (fp_unwrapping.m:66) */
    unwrap1(p + start_col, H, (size_t)W, start_row);
    /* every row from start_col (fp_unwrapping.m:68-70) */
    for (int i = 0; i < H; i++) unwrap1(p + (size_t)i * W, W, 1, start_col);
}
