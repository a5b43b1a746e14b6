// wff_colfft.cu -- WFF2 column sweep with shared-memory FFTs (FP32 form).
//
// Same mathematics as wff_cols_kernel, evaluated in the frequency domain of
// each column.  For one x-frequency plane R_i and one column, with
// h_k(m) = gy(m) e^{j wy_k m} (m in [-s, s]) the truncated, modulated
// window and L >= H + 2s (so the circular convolutions below are the
// linear, zero-boundary ones of the reference):
//     U_k  = IFFT( FFT(R) . H_k )            (|U_k| / (L N) is |sf|)
//     T_k  = U_k . [ |U_k| >= L N thr ],  rows >= H set to 0
//     Ch  += FFT(T_k) . H_k                  (sum over wy_k in the spectrum)
//     C    = IFFT(Ch) / (L^2 N)              (the C_i plane of the direct kernel)
// H_k = FFT(h_k) is tabulated exactly (host, FP64), so the window is the
// reference CPU path's truncated one.  Per column and plane: 1 + 2 nfy + 1
// transforms of length L, all in shared memory / registers; FFT(R) and the
// spectrum accumulator stay in registers for all nfy frequencies.
//
// Transforms: Stockham auto-sort, radix 8/4/2/5/3 stages, ping-pong between
// two shared buffers laid out [L][NC] (NC columns per CTA, column index
// fastest) with one float2 of padding per 16 elements against bank
// conflicts on the strided writes of the early stages.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "glsu_internal.cuh"

namespace glsu {

constexpr int kFftThreads = 512;

// Throughputs of the column-sweep cost model (WffPlan::model_ms), measured
// on GB300: direct kernel in tap-units per second per instantiated
// half-size, FFT sweep in (length x stages) units per second.
constexpr double kModelDirectRate30 = 1.1e13;
constexpr double kModelDirectRate45 = 5.5e12;
constexpr double kModelDirectRate60 = 3.95e12;
constexpr double kModelFftRate = 6.0e11;

struct ColFftPlan {
    int L;
    int nst;
    int radix[12];
};

__device__ __forceinline__ int pidx(int e) { return e + (e >> 4); }

__device__ __forceinline__ float2 cmulf(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// In-register DFTs; INV selects the sign of the exponent (+ for the inverse).
template <bool INV> __device__ __forceinline__ float2 mul_mi(float2 a)
{
    // forward: multiply by -i ; inverse: by +i
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <bool INV> __device__ __forceinline__ void dft2(float2 *v)
{
    const float2 a = v[0], b = v[1];
    v[0] = make_float2(a.x + b.x, a.y + b.y);
    v[1] = make_float2(a.x - b.x, a.y - b.y);
}

template <bool INV> __device__ __forceinline__ void dft4(float2 *v)
{
    const float2 a0 = make_float2(v[0].x + v[2].x, v[0].y + v[2].y);
    const float2 a1 = make_float2(v[0].x - v[2].x, v[0].y - v[2].y);
    const float2 a2 = make_float2(v[1].x + v[3].x, v[1].y + v[3].y);
    const float2 a3 = mul_mi<INV>(make_float2(v[1].x - v[3].x, v[1].y - v[3].y));
    v[0] = make_float2(a0.x + a2.x, a0.y + a2.y);
    v[2] = make_float2(a0.x - a2.x, a0.y - a2.y);
    v[1] = make_float2(a1.x + a3.x, a1.y + a3.y);
    v[3] = make_float2(a1.x - a3.x, a1.y - a3.y);
}

template <bool INV> __device__ __forceinline__ void dft8(float2 *v)
{
    // X[2q] = DFT4(v_r + v_{r+4}), X[2q+1] = DFT4((v_r - v_{r+4}) w8^r)
    const float h = 0.70710678118654752f;
    float2 b[4], c[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        b[r] = make_float2(v[r].x + v[r + 4].x, v[r].y + v[r + 4].y);
        c[r] = make_float2(v[r].x - v[r + 4].x, v[r].y - v[r + 4].y);
    }
    // w8 = e^{-+ i pi/4}
    c[1] = INV ? make_float2(h * (c[1].x - c[1].y), h * (c[1].x + c[1].y))
               : make_float2(h * (c[1].x + c[1].y), h * (c[1].y - c[1].x));
    c[2] = mul_mi<INV>(c[2]);
    c[3] = INV ? make_float2(-h * (c[3].x + c[3].y), h * (c[3].x - c[3].y))
               : make_float2(h * (c[3].y - c[3].x), -h * (c[3].x + c[3].y));
    dft4<INV>(b);
    dft4<INV>(c);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        v[2 * q] = b[q];
        v[2 * q + 1] = c[q];
    }
}

template <bool INV> __device__ __forceinline__ void dft3(float2 *v)
{
    const float s3 = 0.86602540378443865f;  // sin(2 pi / 3)
    const float2 t1 = make_float2(v[1].x + v[2].x, v[1].y + v[2].y);
    const float2 t2 = make_float2(v[1].x - v[2].x, v[1].y - v[2].y);
    const float2 m = make_float2(v[0].x - 0.5f * t1.x, v[0].y - 0.5f * t1.y);
    // forward: X1 = m - i s3 t2, X2 = m + i s3 t2
    const float2 j = INV ? make_float2(-s3 * t2.y, s3 * t2.x) : make_float2(s3 * t2.y, -s3 * t2.x);
    v[0] = make_float2(v[0].x + t1.x, v[0].y + t1.y);
    v[1] = make_float2(m.x + j.x, m.y + j.y);
    v[2] = make_float2(m.x - j.x, m.y - j.y);
}

template <bool INV> __device__ __forceinline__ void dft5(float2 *v)
{
    // X_q = sum_r v_r e^{-+ 2 pi i q r / 5}, via the two symmetric pairs
    const float c1 = 0.30901699437494742f, c2 = -0.80901699437494742f;  // cos(2pi/5), cos(4pi/5)
    const float s1 = 0.95105651629515357f, s2 = 0.58778525229247313f;   // sin(2pi/5), sin(4pi/5)
    const float2 a1 = make_float2(v[1].x + v[4].x, v[1].y + v[4].y);
    const float2 b1 = make_float2(v[1].x - v[4].x, v[1].y - v[4].y);
    const float2 a2 = make_float2(v[2].x + v[3].x, v[2].y + v[3].y);
    const float2 b2 = make_float2(v[2].x - v[3].x, v[2].y - v[3].y);
    const float2 m1 = make_float2(v[0].x + c1 * a1.x + c2 * a2.x, v[0].y + c1 * a1.y + c2 * a2.y);
    const float2 m2 = make_float2(v[0].x + c2 * a1.x + c1 * a2.x, v[0].y + c2 * a1.y + c1 * a2.y);
    // n1 = s1 b1 + s2 b2, n2 = s2 b1 - s1 b2; X1 = m1 -+ i n1, X4 = m1 +- i n1, X2 = m2 -+ i n2, X3 = m2 +- i n2
    const float2 n1 = make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y);
    const float2 n2 = make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y);
    const float2 j1 = INV ? make_float2(-n1.y, n1.x) : make_float2(n1.y, -n1.x);
    const float2 j2 = INV ? make_float2(-n2.y, n2.x) : make_float2(n2.y, -n2.x);
    v[0] = make_float2(v[0].x + a1.x + a2.x, v[0].y + a1.y + a2.y);
    v[1] = make_float2(m1.x + j1.x, m1.y + j1.y);
    v[4] = make_float2(m1.x - j1.x, m1.y - j1.y);
    v[2] = make_float2(m2.x + j2.x, m2.y + j2.y);
    v[3] = make_float2(m2.x - j2.x, m2.y - j2.y);
}

template <int R, bool INV> __device__ __forceinline__ void dft(float2 *v)
{
    if (R == 2) dft2<INV>(v);
    else if (R == 4) dft4<INV>(v);
    else if (R == 8) dft8<INV>(v);
    else if (R == 3) dft3<INV>(v);
    else dft5<INV>(v);
}

// One Stockham stage over all NC columns: in -> out.
template <int R, bool INV, int NC>
__device__ __forceinline__ void fft_stage(const float2 *__restrict__ in, float2 *__restrict__ out, int L, int Ns,
                                          const float2 *__restrict__ tw)
{
    const int LR = L / R;
    const int tstep = L / (Ns * R);
    const int nb = LR * NC;
    for (int b = threadIdx.x; b < nb; b += kFftThreads) {
        const int c = b % NC, j = b / NC;
        const int k = j % Ns;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = in[pidx((j + r * LR) * NC + c)];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; r++) {
                float2 w = __ldg(tw + r * k * tstep);
                if (INV) w.y = -w.y;
                v[r] = cmulf(v[r], w);
            }
        }
        dft<R, INV>(v);
        const int idxD = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; r++) out[pidx((idxD + r * Ns) * NC + c)] = v[r];
    }
}

// Full transform; returns the buffer holding the result (a or b).
template <bool INV, int NC>
__device__ float2 *fft_run(float2 *a, float2 *b, const ColFftPlan &P, const float2 *__restrict__ tw)
{
    int Ns = 1;
    float2 *in = a, *out = b;
    for (int s = 0; s < P.nst; s++) {
        const int R = P.radix[s];
        switch (R) {
        case 8: fft_stage<8, INV, NC>(in, out, P.L, Ns, tw); break;
        case 4: fft_stage<4, INV, NC>(in, out, P.L, Ns, tw); break;
        case 2: fft_stage<2, INV, NC>(in, out, P.L, Ns, tw); break;
        case 5: fft_stage<5, INV, NC>(in, out, P.L, Ns, tw); break;
        default: fft_stage<3, INV, NC>(in, out, P.L, Ns, tw); break;
        }
        __syncthreads();
        Ns *= R;
        float2 *t = in;
        in = out;
        out = t;
    }
    return in;
}

// MAXE: elements (of the L x NC block) owned per thread, upper bound.
// Registers are capped for two CTAs per SM: the stages are bound by shared
// memory and block barriers, and a second CTA hides them (16-19% faster at
// 1024^2 and 2048^2 despite 144-236 bytes of spills a thread).
// A tile-masked run (the surrogate's per-tile fallback) passes the device
// list of needed column groups (list, *list_count); each CTA then walks the
// list with stride gridDim.x.  Without a list, CTA x is column group x.
// Every column is computed the same way in both cases, so a masked run's
// columns equal the full frame's bit for bit.
template <int NC, int MAXE>
__global__ void __launch_bounds__(kFftThreads, 2) wff_colfft_kernel(const float2 *__restrict__ R, float2 *__restrict__ Cout,
                                                                 int H, int pitch, int nfy,
                                                                 const float2 *__restrict__ khat,
                                                                 const float2 *__restrict__ tw, ColFftPlan P,
                                                                 const float *__restrict__ thr_ptr, float LN,
                                                                 float out_scale, const int2 *__restrict__ list,
                                                                 const int *__restrict__ list_count)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = P.L;
    const int nel = L * NC;
    float2 *bufA = reinterpret_cast<float2 *>(smem_raw);
    float2 *bufB = bufA + pidx(nel) + 1;
    const int tid = threadIdx.x;
    const int i = blockIdx.y;
    const size_t plane = (size_t)H * pitch;
    const float2 *Ri = R + i * plane;
    const int nitems = list ? *list_count : (int)gridDim.x;
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    const int x0 = (list ? list[item].x : item) * NC;
    __syncthreads();  // the previous item is done with the shared buffers

    // load the NC columns (rows >= H are zero)
    for (int e = tid; e < nel; e += kFftThreads) {
        const int rho = e / NC, c = e - rho * NC;
        float2 v = make_float2(0.f, 0.f);
        if (rho < H) v = Ri[(size_t)rho * pitch + x0 + c];
        bufA[pidx(e)] = v;
    }
    __syncthreads();
    const float2 *res = fft_run<false, NC>(bufA, bufB, P, tw);
    float2 rh[MAXE], ch[MAXE];
#pragma unroll
    for (int j = 0; j < MAXE; j++) {
        const int e = tid + j * kFftThreads;
        rh[j] = (e < nel) ? res[pidx(e)] : make_float2(0.f, 0.f);
        ch[j] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    const float T = LN * (*thr_ptr);
    const float T2 = T * T;
    for (int k = 0; k < nfy; k++) {
        const float2 *hk = khat + (size_t)k * L;
#pragma unroll
        for (int j = 0; j < MAXE; j++) {
            const int e = tid + j * kFftThreads;
            if (e < nel) bufA[pidx(e)] = cmulf(rh[j], __ldg(hk + e / NC));
        }
        __syncthreads();
        float2 *u = fft_run<true, NC>(bufA, bufB, P, tw);
        // hard threshold in the spatial domain (own elements only)
#pragma unroll
        for (int j = 0; j < MAXE; j++) {
            const int e = tid + j * kFftThreads;
            if (e < nel) {
                const float2 v = u[pidx(e)];
                const bool keep = (e / NC < H) && (v.x * v.x + v.y * v.y >= T2);
                if (!keep) u[pidx(e)] = make_float2(0.f, 0.f);
            }
        }
        __syncthreads();
        float2 *other = (u == bufA) ? bufB : bufA;
        const float2 *sp = fft_run<false, NC>(u, other, P, tw);
#pragma unroll
        for (int j = 0; j < MAXE; j++) {
            const int e = tid + j * kFftThreads;
            if (e < nel) {
                const float2 a = sp[pidx(e)], h = __ldg(hk + e / NC);
                ch[j].x += a.x * h.x - a.y * h.y;
                ch[j].y += a.x * h.y + a.y * h.x;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < MAXE; j++) {
        const int e = tid + j * kFftThreads;
        if (e < nel) bufA[pidx(e)] = ch[j];
    }
    __syncthreads();
    const float2 *cres = fft_run<true, NC>(bufA, bufB, P, tw);
    float2 *Ci = Cout + i * plane;
    for (int e = tid; e < nel; e += kFftThreads) {
        const int rho = e / NC, c = e - rho * NC;
        if (rho < H) {
            const float2 v = cres[pidx(e)];
            Ci[(size_t)rho * pitch + x0 + c] = make_float2(v.x * out_scale, v.y * out_scale);
        }
    }
    }  // items
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// Stage radices of a length-n transform in one of three orders (the tuner's
// radix-plan knob): 0 = 8, 4, 2 then 5, 3; 1 = 4, 2 then 5, 3 (no radix 8);
// 2 = 5, 3 first, then 8, 4, 2.  Returns the stage count, or -1 when n has a
// prime factor above 5.
static int factor(int n, int *rad, int order = 0)
{
    int ns = 0;
    auto take = [&](int r) {
        while (n % r == 0 && ns < 12) {
            rad[ns++] = r;
            n /= r;
        }
    };
    if (order == 2) {
        take(5);
        take(3);
    }
    if (order != 1) take(8);
    take(4);
    take(2);
    take(5);
    take(3);
    return n == 1 ? ns : -1;
}

// Transform lengths L >= need (up to 2 need + 16) whose stages factor, in
// increasing cost L x number of stages (ties: the shorter); at most n of them.
static int length_candidates(int need, int *out, int n)
{
    std::vector<std::pair<long, int>> c;
    for (int L = need; L <= 2 * need + 16; L++) {
        int rad[12];
        const int ns = factor(L, rad);
        if (ns >= 1 && ns <= 12) c.push_back({(long)L * ns, L});
    }
    std::sort(c.begin(), c.end());
    int k = 0;
    for (; k < n && k < (int)c.size(); k++) out[k] = c[k].second;
    return k;
}

static int colfft_nc(int L) { return L <= 1600 ? 4 : 2; }
static bool colfft_fits(int L, int nc, int pitch)
{
    const int nel = L * nc;
    return (nc == 4 || nc == 2) && (size_t)nel <= (size_t)kFftThreads * 13 && pitch % nc == 0 &&
           sizeof(float2) * 2 * (size_t)(nel + (nel >> 4) + 1) <= 112 * 1024;
}

int WffPlan::init_colfft()
{
    if (prec != GLSU_F32) return GLSU_OK;
    int L;
    if (length_candidates(H + 2 * sy, &L, 1) < 1) return GLSU_OK;  // no suitable length: direct kernel
    if (!colfft_fits(L, colfft_nc(L), pitch)) return GLSU_OK;      // registers per thread, shared memory
    return build_colfft(L);
}

// Tables of the FFT sweep for transform length L (replacing any others), with
// the default plan variant: H_k = DFT of h_k(m) = gy(m) e^{j wy_k m},
// m in [-sy, sy] placed circularly, and the twiddles e^{-2 pi i t / L}.
int WffPlan::build_colfft(int L)
{
    if (prec != GLSU_F32 || L < H + 2 * sy || !colfft_fits(L, colfft_nc(L), pitch))
        return fail(GLSU_ERR_UNSUPPORTED, "no shared-memory FFT plan of that length for this handle");
    int rad[12];
    const int ns = factor(L, rad);
    if (ns < 1 || ns > 12) return fail(GLSU_ERR_UNSUPPORTED, "transform length has a prime factor above 5");
    release_colfft();
    std::vector<float> kh(2 * (size_t)nfy * L), tw(2 * (size_t)L);
    for (int k = 0; k < nfy; k++) {
        const double wy = this->p.wyl + (double)k * this->p.wyi;
        for (int w = 0; w < L; w++) {
            double re = 0, im = 0;
            for (int m = -sy; m <= sy; m++) {
                const double ang = wy * m - 2.0 * M_PI * (double)w * (double)m / (double)L;
                re += gy[m + sy] * std::cos(ang);
                im += gy[m + sy] * std::sin(ang);
            }
            kh[2 * ((size_t)k * L + w)] = (float)re;
            kh[2 * ((size_t)k * L + w) + 1] = (float)im;
        }
    }
    for (int t = 0; t < L; t++) {
        tw[2 * t] = (float)std::cos(-2.0 * M_PI * t / L);
        tw[2 * t + 1] = (float)std::sin(-2.0 * M_PI * t / L);
    }
    if (cudaMalloc(&d_khat, kh.size() * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&d_tw, tw.size() * sizeof(float)) != cudaSuccess) {
        release_colfft();
        return fail(GLSU_ERR_ALLOC, "cudaMalloc of the column FFT tables failed");
    }
    GLSU_CUDA_TRY(cudaMemcpy(d_khat, kh.data(), kh.size() * sizeof(float), cudaMemcpyHostToDevice));
    GLSU_CUDA_TRY(cudaMemcpy(d_tw, tw.data(), tw.size() * sizeof(float), cudaMemcpyHostToDevice));
    fft_L = L;
    return set_fft_plan(colfft_nc(L), 0);
}

int fft_length_candidates(const WffPlan &P, int *out, int n)
{
    if (P.prec != GLSU_F32 || P.fft_L == 0) return 0;
    return length_candidates(P.H + 2 * P.sy, out, n);
}

int WffPlan::set_fft_plan(int nc, int order)
{
    if (fft_L == 0) return fail(GLSU_ERR_UNSUPPORTED, "no shared-memory FFT plan for this handle");
    if (order < 0 || order > 2 || !colfft_fits(fft_L, nc, pitch))
        return fail(GLSU_ERR_UNSUPPORTED, "FFT plan variant does not fit this transform length");
    int rad[12];
    const int ns = factor(fft_L, rad, order);
    if (ns < 1 || ns > 12) return fail(GLSU_ERR_UNSUPPORTED, "transform length does not factor in that order");
    fft_nc = nc;
    fft_order = order;
    fft_nst = ns;
    for (int k = 0; k < ns; k++) fft_radix[k] = rad[k];
    return GLSU_OK;
}

void WffPlan::release_colfft()
{
    cudaFree(d_khat);
    cudaFree(d_tw);
    d_khat = d_tw = nullptr;
    fft_L = 0;
}

template <int NC, int MAXE> static int launch_colfft_t(const WffPlan &P, cudaStream_t s)
{
    ColFftPlan cp;
    cp.L = P.fft_L;
    cp.nst = P.fft_nst;
    for (int k = 0; k < 12; k++) cp.radix[k] = k < P.fft_nst ? P.fft_radix[k] : 0;
    const int nel = cp.L * NC;
    const size_t smem = sizeof(float2) * 2 * (size_t)(nel + (nel >> 4) + 1);
    GLSU_TRY(raise_smem_limit((const void *)wff_colfft_kernel<NC, MAXE>, 112 * 1024));
    if (smem > 112 * 1024) return fail(GLSU_ERR_UNSUPPORTED, "column FFT length too large");
    const double N = 1.0 / P.inv_norm;
    const int ngroups = P.pitch / NC;
    dim3 grid(ngroups, P.nfx);
    const int2 *list = nullptr;
    const int *count = nullptr;
    if (P.mask.flags) {
        // tile-masked run: the column groups whose columns, grown by sx,
        // meet a flagged tile (all rows: a column's transform spans them)
        if (!P.d_list) return fail(GLSU_ERR_INVALID, "tile-masked run without a tile list buffer");
        TileMask m = P.mask;
        m.my = 0;
        m.mx = P.sx;
        GLSU_TRY(launch_mask_list(m, ngroups, 1, P.H, NC, P.d_list, P.d_list_count, s));
        list = P.d_list;
        count = P.d_list_count;
        grid.x = std::max(1, std::min(ngroups, (2 * device_sm_count() + P.nfx - 1) / P.nfx));
    }
    wff_colfft_kernel<NC, MAXE><<<grid, kFftThreads, smem, s>>>(
        (const float2 *)P.d_R, (float2 *)P.d_C, P.H, P.pitch, P.nfy, (const float2 *)P.d_khat,
        (const float2 *)P.d_tw, cp, (const float *)P.d_thr, (float)(cp.L * N),
        (float)(1.0 / ((double)cp.L * cp.L * N)), list, count);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

int launch_colfft(const WffPlan &P, cudaStream_t s)
{
    const int nc = P.fft_nc;
    const int per = (P.fft_L * nc + kFftThreads - 1) / kFftThreads;  // elements owned per thread
    if (nc == 4) {
        if (per <= 3) return launch_colfft_t<4, 3>(P, s);
        if (per <= 5) return launch_colfft_t<4, 5>(P, s);
        if (per <= 10) return launch_colfft_t<4, 10>(P, s);
        return launch_colfft_t<4, 13>(P, s);
    }
    if (per <= 10) return launch_colfft_t<2, 10>(P, s);
    return launch_colfft_t<2, 13>(P, s);
}

// ---------------------------------------------------------------------------
// autotuner
// ---------------------------------------------------------------------------
// GLSU_METHOD_AUTO (the default) decides from the shape alone, with a cost
// model of the two column sweeps (model_ms below), so that the same inputs
// give the same bits in every process and on every box.  The timed search
// below runs only on request (GLSU_METHOD_TIMED, or GLSU_AUTOTUNE=time in
// the environment).
//
// Timed search.  Candidates: the direct column kernel, and the FFT sweep at the three
// cheapest transform lengths (L x stages), then, at the fastest length, with
// 4 or 2 columns per CTA and each radix order.  Each is launched once
// (warm-up), then twice between CUDA events on the plan's own buffers; the
// kernels have no data-dependent control flow, so the buffers' contents do
// not matter.  The FFT is taken only when at least 10% faster than the
// direct kernel, so that near ties keep the direct kernel, and the plan
// variants are tried only when the best length is within 1.5x of it.  Results are kept
// per shape for the process, so every handle of a shape runs the same
// kernels.  GLSU_AUTOTUNE=0 in the environment skips the timing (the direct
// kernel).
namespace {
struct TuneKey {
    int v[9];
    bool operator<(const TuneKey &o) const { return std::lexicographical_compare(v, v + 9, o.v, o.v + 9); }
};
struct TuneResult {
    int method, L, nc, order;
    float ms_direct, ms_fft;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneResult> g_tune;
}  // namespace

// Modelled device time (ms) of one full-frame column sweep of this plan.
// Direct kernel: per output pixel, x-frequency and y-frequency, two column
// filters of 2S+1 taps (S the instantiated half-size), the first one also
// over the 2S-row halo of each 128-row tile, at a rate per instantiation.
// FFT sweep: per column and x-frequency, 2 nfy + 2 transforms of length L
// with nst stages, at a rate scaled down when a CTA's L x columns elements
// leave its 512 threads short of work.  The rates are GB300 measurements
// (2070 MHz) of both kernels at 256^2 .. 2048^2.
double WffPlan::model_ms(int m) const
{
    if (m == GLSU_METHOD_FFT) {
        if (fft_L == 0) return 1e30;
        const double units = (double)pitch * nfx * (2.0 * nfy + 2.0) * fft_L * fft_nst;
        const double fill = std::min(1.0, (double)fft_L * fft_nc / (kFftThreads * 8.0));
        return units / (kModelFftRate * fill) * 1e3;
    }
    const int S = syi;
    const double taps = (2.0 * S + 1.0) * (2.0 + 2.0 * S / 128.0);
    const double rate = S <= 30 ? kModelDirectRate30 : (S <= 45 ? kModelDirectRate45 : kModelDirectRate60);
    return (double)pitch * H * nfx * nfy * taps / rate * 1e3;
}

// AUTO without timing: the transform length cheapest by L x stages (built
// by init_colfft), the default plan variant, and the FFT sweep when its
// modelled time is below 0.9 x the direct kernel's.
int WffPlan::choose_by_model()
{
    auto_method = GLSU_METHOD_DIRECT;
    if (prec != GLSU_F32 || fft_L == 0 || d_khat == nullptr) return GLSU_OK;
    int L;
    if (length_candidates(H + 2 * sy, &L, 1) == 1 && L != fft_L) GLSU_TRY(build_colfft(L));
    GLSU_TRY(set_fft_plan(colfft_nc(fft_L), 0));
    tune_ms_direct = (float)model_ms(GLSU_METHOD_DIRECT);
    tune_ms_fft = (float)model_ms(GLSU_METHOD_FFT);
    if (tune_ms_fft < 0.9f * tune_ms_direct) auto_method = GLSU_METHOD_FFT;
    return GLSU_OK;
}

int WffPlan::autotune(cudaStream_t s)
{
    tuned = true;
    timed = false;
    auto_method = GLSU_METHOD_DIRECT;
    tune_ms_direct = tune_ms_fft = 0;
    if (prec != GLSU_F32 || fft_L == 0 || d_khat == nullptr) return GLSU_OK;
    const char *env = std::getenv("GLSU_AUTOTUNE");
    if (env && env[0] == '0') return GLSU_OK;
    const bool want_timing = method == GLSU_METHOD_TIMED || (env && std::strcmp(env, "time") == 0);
    if (!want_timing) return choose_by_model();
    timed = true;
    const TuneKey key{{W, H, pitch, sx, sy, nfx, nfy, H + 2 * sy, (int)(1000 * p.wyl + 0.5)}};
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(key);
    if (it == g_tune.end()) {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
            if (e0) cudaEventDestroy(e0);
            return fail(GLSU_ERR_CUDA, "cudaEventCreate failed");
        }
        const int saved = method;
        int rc = GLSU_OK;
        auto time_it = [&](int m, float *ms) {
            method = m;
            for (int k = 0; k < 3 && rc == GLSU_OK; k++) {
                if (k == 1 && cudaEventRecord(e0, s) != cudaSuccess) rc = fail(GLSU_ERR_CUDA, "cudaEventRecord");
                if (rc == GLSU_OK) rc = launch_column_sweep(*this, s);
            }
            if (rc == GLSU_OK && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                                  cudaEventElapsedTime(ms, e0, e1) != cudaSuccess))
                rc = fail(GLSU_ERR_CUDA, "timing a column-sweep candidate failed");
            *ms *= 0.5f;
        };
        TuneResult r{GLSU_METHOD_DIRECT, fft_L, fft_nc, fft_order, 0.f, 0.f};
        time_it(GLSU_METHOD_DIRECT, &r.ms_direct);
        float best = -1.f;
        int lens[3];
        const int nl = length_candidates(H + 2 * sy, lens, 3);
        for (int j = 0; j < nl && rc == GLSU_OK; j++) {
            if (build_colfft(lens[j]) != GLSU_OK) continue;
            float ms = 0;
            time_it(GLSU_METHOD_FFT, &ms);
            if (rc == GLSU_OK && (best < 0 || ms < best)) {
                best = ms;
                r.L = lens[j];
                r.nc = fft_nc;
                r.order = fft_order;
            }
        }
        if (rc == GLSU_OK && r.L != fft_L) rc = build_colfft(r.L);
        const int nc0 = fft_nc;
        for (int nc : {nc0, 6 - nc0}) {
            if (rc != GLSU_OK || best < 0 || best > 1.5f * r.ms_direct) break;
            for (int order = 0; order < 3 && rc == GLSU_OK; order++) {
                if ((nc == nc0 && order == 0) || set_fft_plan(nc, order) != GLSU_OK) continue;
                float ms = 0;
                time_it(GLSU_METHOD_FFT, &ms);
                if (rc == GLSU_OK && ms < best) {
                    best = ms;
                    r.nc = nc;
                    r.order = order;
                }
            }
        }
        set_error(std::string());  // variants that did not fit leave no message
        method = saved;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc != GLSU_OK) return rc;
        r.ms_fft = best;
        if (best > 0 && best < 0.9f * r.ms_direct) r.method = GLSU_METHOD_FFT;
        it = g_tune.emplace(key, r).first;
    }
    const TuneResult &r = it->second;
    auto_method = r.method;
    tune_ms_direct = r.ms_direct;
    tune_ms_fft = r.ms_fft;
    if (r.L != fft_L) GLSU_TRY(build_colfft(r.L));
    return set_fft_plan(r.nc, r.order);
}

}  // namespace glsu
