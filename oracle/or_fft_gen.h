/*
 * or_fft_gen.h -- the oracle's mixed-radix Stockham FFT, generated for one
 * element type.  TEST INFRASTRUCTURE ONLY (see glsu_oracle.c).
 *
 * Before including, define OR_REAL (double or float) and OR_FN(name), the
 * name of each generated type and function (e.g. name##_f).  Twiddles are
 * computed in double and rounded to OR_REAL once; all arithmetic is OR_REAL.
 */
/* ------------------------------------------------------------------------ */
/* Mixed-radix Stockham FFT (complex OR_REAL, interleaved re/im).           */
/* ------------------------------------------------------------------------ */
typedef struct {
    int n;
    int nf;
    int fac[40];
    OR_REAL *w; /* w[2t], w[2t+1] = cos, sin of (-2 pi t / n) */
} OR_FN(fft_plan);

static int OR_FN(fft_plan_init)(OR_FN(fft_plan) *p, int n)
{
    p->n = n;
    p->nf = 0;
    int t = n;
    while (t % 4 == 0) { p->fac[p->nf++] = 4; t /= 4; }
    while (t % 2 == 0) { p->fac[p->nf++] = 2; t /= 2; }
    for (int r = 3; t > 1; r += 2) {
        if (r > 64) return -1; /* radices above 64 are not supported */
        while (t % r == 0) { p->fac[p->nf++] = r; t /= r; }
    }
    p->w = (OR_REAL *)malloc(sizeof(OR_REAL) * 2 * (size_t)n);
    if (!p->w) return -1;
    for (int i = 0; i < n; i++) {
        double a = -2.0 * M_PI * (double)i / (double)n;
        p->w[2 * i] = (OR_REAL)cos(a);
        p->w[2 * i + 1] = (OR_REAL)sin(a);
    }
    return 0;
}

static void OR_FN(fft_plan_free)(OR_FN(fft_plan) *p)
{
    free(p->w);
    p->w = NULL;
}

/* One transform of length p->n.  x and y are 2n-OR_REAL buffers; the result
 * ends in x.  inverse != 0 computes the unnormalised backward transform. */
static void OR_FN(fft_exec)(const OR_FN(fft_plan) *p, OR_REAL *x, OR_REAL *y, int inverse)
{
    const int n = p->n;
    if (n == 1) return;
    const OR_REAL sgn = inverse ? -1.0 : 1.0; /* sign applied to sin() */
    OR_REAL *in = x, *out = y;
    int Ns = 1;
    OR_REAL vr[64], vi[64], tr[64], ti[64];
    for (int s = 0; s < p->nf; s++) {
        const int R = p->fac[s];
        const int nR = n / R;
        const int tstep = n / (Ns * R);
        for (int j = 0; j < nR; j++) {
            const int k = j % Ns;
            for (int r = 0; r < R; r++) {
                vr[r] = in[2 * (j + r * nR)];
                vi[r] = in[2 * (j + r * nR) + 1];
            }
            if (Ns > 1) {
                for (int r = 1; r < R; r++) {
                    const int e = r * k * tstep; /* < R Ns tstep = n */
                    OR_REAL c = p->w[2 * e], sn = sgn * p->w[2 * e + 1];
                    OR_REAL a = vr[r] * c - vi[r] * sn;
                    OR_REAL b = vr[r] * sn + vi[r] * c;
                    vr[r] = a;
                    vi[r] = b;
                }
            }
            if (R == 2) {
                OR_REAL ar = vr[0] + vr[1], ai = vi[0] + vi[1];
                OR_REAL br = vr[0] - vr[1], bi = vi[0] - vi[1];
                tr[0] = ar; ti[0] = ai; tr[1] = br; ti[1] = bi;
            } else if (R == 4) {
                OR_REAL s0r = vr[0] + vr[2], s0i = vi[0] + vi[2];
                OR_REAL d0r = vr[0] - vr[2], d0i = vi[0] - vi[2];
                OR_REAL s1r = vr[1] + vr[3], s1i = vi[1] + vi[3];
                OR_REAL d1r = vr[1] - vr[3], d1i = vi[1] - vi[3];
                /* forward: multiply d1 by -i ; inverse: by +i */
                OR_REAL mr = sgn * d1i, mi = -sgn * d1r;
                tr[0] = s0r + s1r; ti[0] = s0i + s1i;
                tr[2] = s0r - s1r; ti[2] = s0i - s1i;
                tr[1] = d0r + mr;  ti[1] = d0i + mi;
                tr[3] = d0r - mr;  ti[3] = d0i - mi;
            } else {
                const int step = n / R;
                for (int q = 0; q < R; q++) {
                    OR_REAL sr = 0, si = 0;
                    int qr = 0; /* (q r) mod R */
                    for (int r = 0; r < R; r++, qr = (qr + q >= R) ? qr + q - R : qr + q) {
                        const int e = qr * step;
                        OR_REAL c = p->w[2 * e], sn = sgn * p->w[2 * e + 1];
                        sr += vr[r] * c - vi[r] * sn;
                        si += vr[r] * sn + vi[r] * c;
                    }
                    tr[q] = sr;
                    ti[q] = si;
                }
            }
            const int idxD = (j / Ns) * Ns * R + k;
            for (int r = 0; r < R; r++) {
                out[2 * (idxD + r * Ns)] = tr[r];
                out[2 * (idxD + r * Ns) + 1] = ti[r];
            }
        }
        OR_REAL *t = in; in = out; out = t;
        Ns *= R;
    }
    if (in != x) memcpy(x, in, sizeof(OR_REAL) * 2 * (size_t)n);
}

/* 2D transform of an H x W row-major plane, in place.  Columns are moved
 * through the scratch in blocks of OR_COLBLK (whole cache lines of the
 * plane), then transformed one by one. */
#ifndef OR_COLBLK
#define OR_COLBLK 8
#endif
typedef struct {
    OR_FN(fft_plan) row, col;
    OR_REAL *buf, *scr; /* buf: 2 * OR_COLBLK * H; scr: 2 * max(W, H) */
} OR_FN(fft2_plan);

static int OR_FN(fft2_init)(OR_FN(fft2_plan) *p, int W, int H)
{
    if (OR_FN(fft_plan_init)(&p->row, W)) return -1;
    if (OR_FN(fft_plan_init)(&p->col, H)) return -1;
    int m = W > H ? W : H;
    p->buf = (OR_REAL *)malloc(sizeof(OR_REAL) * 2 * (size_t)OR_COLBLK * (size_t)H);
    p->scr = (OR_REAL *)malloc(sizeof(OR_REAL) * 2 * (size_t)m);
    return (p->buf && p->scr) ? 0 : -1;
}

static void OR_FN(fft2_free)(OR_FN(fft2_plan) *p)
{
    OR_FN(fft_plan_free)(&p->row);
    OR_FN(fft_plan_free)(&p->col);
    free(p->buf);
    free(p->scr);
}

static void OR_FN(fft2_exec)(OR_FN(fft2_plan) *p, OR_REAL *a, int inverse)
{
    const int W = p->row.n, H = p->col.n;
    for (int i = 0; i < H; i++) {
        OR_REAL *r = a + 2 * (size_t)i * W;
        OR_FN(fft_exec)(&p->row, r, p->scr, inverse);
    }
    for (int j0 = 0; j0 < W; j0 += OR_COLBLK) {
        const int nb = W - j0 < OR_COLBLK ? W - j0 : OR_COLBLK;
        for (int i = 0; i < H; i++) {
            const OR_REAL *src = a + 2 * ((size_t)i * W + j0);
            for (int b = 0; b < nb; b++) {
                p->buf[2 * ((size_t)b * H + i)] = src[2 * b];
                p->buf[2 * ((size_t)b * H + i) + 1] = src[2 * b + 1];
            }
        }
        for (int b = 0; b < nb; b++) OR_FN(fft_exec)(&p->col, p->buf + 2 * (size_t)b * H, p->scr, inverse);
        for (int i = 0; i < H; i++) {
            OR_REAL *dst = a + 2 * ((size_t)i * W + j0);
            for (int b = 0; b < nb; b++) {
                dst[2 * b] = p->buf[2 * ((size_t)b * H + i)];
                dst[2 * b + 1] = p->buf[2 * ((size_t)b * H + i) + 1];
            }
        }
    }
}

