// wfr_kernels.cu -- WFR2, windowed Fourier ridges, on sm_103a.
//
// The reference (CPU: WFT/WFT2_CPU.cpp:391-694; CUDA: WFT/WFT2_CUDAf.cu:
// 1174-1319) computes, for every frequency (wx, wy) of the grid,
//     sf = f (*) (g e^{j(wx x + wy y)})      (g: the L2-normalised window)
// and keeps per pixel the largest |sf| (the ridge r), its wx, wy and
// angle(sf); then the curvature least squares
//     cxx = -conv2(wx, x.*g, 'same') / sum(x.*x.*g)   (map replicated
//     cyy = -conv2(wy, y.*g, 'same') / sum(y.*y.*g)    beyond the border),
// the compensated phase phase - atan(sx^2 cxx)/2 - atan(sy^2 cyy)/2 and the
// amplitude b.  Same formulation as the CPU reference (truncated window), on
// the WFF2 sweep engine of wff_kernels.cu:
//   1. the WFF2 row pass (wff_rows_demod_kernel) gives the planes
//      R_i = (f e^{-j wx_i x}) (*)_x gx for every wx_i;
//   2. wfr_cols_kernel, one CTA per (32-column tile, TY rows, wx_i): one TMA
//      load of R_i rows y0 - s .. y0 + TY + s, then for every wy_k the first
//      column filter U = (R_i e^{-j wy_k y}) (*)_y gy / norm, with
//      sf = U e^{+j(wx x + wy y)}, |sf| = |U|; each output row keeps its
//      arg-max over wy in registers (ties: the later wy) and writes |sf|,
//      the wy index and angle(sf) into the partial planes of wx_i;
//   3. wfr_reduce_kernel: per pixel the arg-max over wx_i of (|sf|, wy
//      index, wx index) -- the frequency that the reference's wy-major,
//      wx-minor loop with `>=` leaves (:505-518);
//   4. wfr_curv_rows_kernel / wfr_final_kernel: the two curvature
//      convolutions separably (rows with n gx(n) and gx(n), columns with
//      gy(m) and m gy(m), indices clamped to the image), then cxx, cyy,
//      phase_comp, b (:674-692).
#include <algorithm>
#include <cmath>

#include "glsu_internal.cuh"
#include "ptx_sm103.cuh"
#include "wff_common.cuh"

namespace glsu {

template <typename T, int S> struct WfrGeom {
    static constexpr int WARPS = 8;
    static constexpr int THREADS = 32 * WARPS;
    static constexpr int TY = (sizeof(T) == 4) ? (S <= 30 ? 128 : 64) : (S <= 20 ? 64 : 32);  // output rows per CTA
    static constexpr int KC = TY / WARPS;                    // output rows per warp
    static constexpr int ROWS_R = TY + 2 * S;                // rows of R needed
    static constexpr int BOX = (sizeof(T) == 4) ? 64 : 16;   // rows per TMA box (the plan's map)
    static constexpr int NBOX = (ROWS_R + BOX - 1) / BOX;
    static constexpr int RT = NBOX * BOX;
    static constexpr int FPC = (int)(sizeof(C2<T>) / 4);
    static constexpr uint32_t TX_BYTES = (uint32_t)(NBOX * BOX * 32 * sizeof(C2<T>));
    static constexpr size_t SMEM = sizeof(C2<T>) * (size_t)RT * 32 + 16;
    static_assert(SMEM <= 227 * 1024, "WFR column tile exceeds shared memory");
};

template <typename T> __device__ __forceinline__ T mag_key(C2<T> a);
template <> __device__ __forceinline__ float mag_key<float>(float2 a) { return a.x * a.x + a.y * a.y; }
template <> __device__ __forceinline__ double mag_key<double>(double2 a) { return sqrt(a.x * a.x + a.y * a.y); }
__device__ __forceinline__ float mag_of_key(float k) { return sqrtf(k); }
__device__ __forceinline__ double mag_of_key(double k) { return k; }
__device__ __forceinline__ float atan2_t(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ double atan2_t(double y, double x) { return atan2(y, x); }

template <typename T, int S>
__global__ void __launch_bounds__(WfrGeom<T, S>::THREADS, 1)
    wfr_cols_kernel(const __grid_constant__ CUtensorMap tmR, const C2<T> *__restrict__ ex,
                    const C2<T> *__restrict__ ey, int nfy, int W, int H, int pitch, Taps<T, S> gA,
                    T *__restrict__ pabs, int *__restrict__ pk, T *__restrict__ pph, int *__restrict__ err)
{
    using G = WfrGeom<T, S>;
    extern __shared__ __align__(1024) unsigned char smem_wfr[];
    C2<T> *Rt = reinterpret_cast<C2<T> *>(smem_wfr);
    uint64_t *bar = reinterpret_cast<uint64_t *>(Rt + G::RT * 32);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * G::TY, i = blockIdx.z;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        mbar_expect_tx(bar, G::TX_BYTES);
#pragma unroll 1
        for (int b = 0; b < G::NBOX; b++)
            tma_load_3d(Rt + b * G::BOX * 32, &tmR, bar, x0 * G::FPC, y0 - S + b * G::BOX, i);
    }
    const bool late = !mbar_wait_bounded(bar, 0);
    if (__syncthreads_or(late)) {
        if (tid == 0) {
            atomicExch(err, GLSU_ERR_TIMEOUT);
            mbar_wait_bounded(bar, 0);  // let copies still in flight land before exit
        }
        return;
    }

    const size_t eys = (size_t)H + 2 * kPhasorPad;
    const int q0 = w * G::KC;  // R row (from y0 - S) of the first tap of this warp's first output row
    T best[G::KC];
    int bk[G::KC];
#pragma unroll
    for (int kk = 0; kk < G::KC; kk++) {
        best[kk] = -1;
        bk[kk] = 0;
    }
    for (int k = 0; k < nfy; k++) {
        const C2<T> *eyk = ey + k * eys + kPhasorPad;
        C2<T> a[G::KC];
#pragma unroll
        for (int kk = 0; kk < G::KC; kk++) a[kk] = mk<T>(0, 0);
#pragma unroll
        for (int j = 0; j < G::KC + 2 * S; j++) {
            const int q = q0 + j;
            const C2<T> r = Rt[q * 32 + lane];
            int gr = y0 - S + q;
            gr = min(max(gr, -kPhasorPad), H - 1 + kPhasorPad);
            const C2<T> p = __ldg(eyk + gr);
            const C2<T> d = mk<T>(r.x * p.x - r.y * p.y, r.x * p.y + r.y * p.x);
#pragma unroll
            for (int kk = 0; kk < G::KC; kk++) {
                const int m = j - kk;
                if (m >= 0 && m <= 2 * S) cfma(a[kk], gA.g[m], d);
            }
        }
#pragma unroll
        for (int kk = 0; kk < G::KC; kk++) {
            const T key = mag_key<T>(a[kk]);
            if (key >= best[kk]) {  // the later wy wins ties
                best[kk] = key;
                bk[kk] = k;
            }
        }
    }

    const int x = x0 + lane;
    if (x >= W) return;
    const size_t exs = (size_t)pitch + 2 * kPhasorPad;
    const C2<T> e1 = __ldg(ex + i * exs + kPhasorPad + x);  // e^{-j wx x}
    const size_t N = (size_t)H * W;
#pragma unroll
    for (int kk = 0; kk < G::KC; kk++) {
        const int y = y0 + q0 + kk;
        if (y >= H) break;
        // U at the winning wy again (the same taps in the same order as in the sweep)
        const C2<T> *eyk = ey + bk[kk] * eys + kPhasorPad;
        C2<T> u = mk<T>(0, 0);
#pragma unroll 1
        for (int m = 0; m <= 2 * S; m++) {
            const int q = q0 + kk + m;
            const C2<T> r = Rt[q * 32 + lane];
            int gr = y0 - S + q;
            gr = min(max(gr, -kPhasorPad), H - 1 + kPhasorPad);
            const C2<T> p = __ldg(eyk + gr);
            cfma(u, gA.g[m], mk<T>(r.x * p.x - r.y * p.y, r.x * p.y + r.y * p.x));
        }
        const C2<T> e2 = __ldg(eyk + y);  // e^{-j wy y}
        // sf = U conj(e1) conj(e2)
        const T ar = u.x * e1.x + u.y * e1.y, ai = u.y * e1.x - u.x * e1.y;
        const T sr = ar * e2.x + ai * e2.y, si = ai * e2.x - ar * e2.y;
        const size_t o = (size_t)i * N + (size_t)y * W + x;
        pabs[o] = mag_of_key(best[kk]);
        pk[o] = bk[kk];
        pph[o] = atan2_t(si, sr);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) wfr_reduce_kernel(const T *__restrict__ pabs, const int *__restrict__ pk,
                                                         const T *__restrict__ pph, int nfx, int H, int W,
                                                         double wxl, double wxi, double wyl, double wyi,
                                                         T *__restrict__ r, T *__restrict__ wx, T *__restrict__ wy,
                                                         T *__restrict__ ph)
{
    const size_t N = (size_t)H * W;
    for (int row = blockIdx.x; row < H; row += gridDim.x)
        for (int x = threadIdx.x; x < W; x += blockDim.x) {
            const size_t p = (size_t)row * W + x;
            T best = -1, bp = 0;
            int bk = 0, bi = 0;
            for (int i = 0; i < nfx; i++) {
                const T a = pabs[(size_t)i * N + p];
                const int k = pk[(size_t)i * N + p];
                // wy-major, wx-minor order with `>=`: equal magnitudes go to the
                // larger wy index, then (i ascending) to the larger wx index
                if (a > best || (a == best && k >= bk)) {
                    best = a;
                    bk = k;
                    bi = i;
                    bp = pph[(size_t)i * N + p];
                }
            }
            r[p] = best;
            wx[p] = (T)(wxl + (double)bi * wxi);
            wy[p] = (T)(wyl + (double)bk * wyi);
            ph[p] = bp;
        }
}

// Curvature taps: gx[n + sx] = e^{-n^2 / 2 sx^2} (unnormalised; the 2-D
// normalisation cancels in cxx, cyy).
struct WfrCurvTaps {
    double gx[2 * kMaxHalf + 1], gy[2 * kMaxHalf + 1];
    int sx, sy;
};

// A(y, x) = sum_n n gx(n) wx(y, x - n), B(y, x) = sum_n gx(n) wy(y, x - n),
// column indices clamped to the image.
template <typename T>
__global__ void __launch_bounds__(256) wfr_curv_rows_kernel(const T *__restrict__ wx, const T *__restrict__ wy,
                                                            int H, int W, const __grid_constant__ WfrCurvTaps tp,
                                                            T *__restrict__ A, T *__restrict__ B)
{
    for (int row = blockIdx.x; row < H; row += gridDim.x)
        for (int x = threadIdx.x; x < W; x += blockDim.x) {
            const T *wxr = wx + (size_t)row * W, *wyr = wy + (size_t)row * W;
            T a = 0, b = 0;
            for (int n = -tp.sx; n <= tp.sx; n++) {
                const int xi = min(max(x - n, 0), W - 1);
                const T g = (T)tp.gx[n + tp.sx];
                a += (T)n * g * wxr[xi];
                b += g * wyr[xi];
            }
            A[(size_t)row * W + x] = a;
            B[(size_t)row * W + x] = b;
        }
}

template <typename T> __device__ __forceinline__ T atan_t(T v);
template <> __device__ __forceinline__ float atan_t<float>(float v) { return atanf(v); }
template <> __device__ __forceinline__ double atan_t<double>(double v) { return atan(v); }
template <typename T> __device__ __forceinline__ T pow_t(T a, T b);
template <> __device__ __forceinline__ float pow_t<float>(float a, float b) { return powf(a, b); }
template <> __device__ __forceinline__ double pow_t<double>(double a, double b) { return pow(a, b); }

// Columns of the two convolutions (row indices clamped), then cxx, cyy, the
// compensated phase and the amplitude.
template <typename T>
__global__ void __launch_bounds__(256) wfr_final_kernel(const T *__restrict__ A, const T *__restrict__ B, int H,
                                                        int W, const __grid_constant__ WfrCurvTaps tp, double dx,
                                                        double dy, double sigx, double sigy,
                                                        const T *__restrict__ r, const T *__restrict__ ph,
                                                        T *__restrict__ cxx, T *__restrict__ cyy,
                                                        T *__restrict__ phc, T *__restrict__ b)
{
    for (int row = blockIdx.x; row < H; row += gridDim.x)
        for (int x = threadIdx.x; x < W; x += blockDim.x) {
            T sa = 0, sb = 0;
            for (int m = -tp.sy; m <= tp.sy; m++) {
                const int yi = min(max(row - m, 0), H - 1);
                const T g = (T)tp.gy[m + tp.sy];
                sa += g * A[(size_t)yi * W + x];
                sb += (T)m * g * B[(size_t)yi * W + x];
            }
            const size_t p = (size_t)row * W + x;
            const T cx = -sa / (T)dx, cy = -sb / (T)dy;
            const T s2x = (T)(sigx * sigx), s2y = (T)(sigy * sigy);
            T pc = ph[p] - (T)0.5 * atan_t<T>(s2x * cx) - (T)0.5 * atan_t<T>(s2y * cy);
            pc = atan2_t(sin(pc), cos(pc));
            const T q = (T)(0.25 / M_PI);
            const T bb = r[p] * pow_t<T>((1 + s2x * s2x * cx * cx) * q / s2x, (T)0.25) *
                         pow_t<T>((1 + s2y * s2y * cy * cy) * q / s2y, (T)0.25);
            cxx[p] = cx;
            cyy[p] = cy;
            phc[p] = pc;
            b[p] = bb;
        }
}

template <typename T, int S>
static int launch_wfr_cols(const WffPlan &P, const WfrBuffers &wb, cudaStream_t s)
{
    using G = WfrGeom<T, S>;
    GLSU_TRY(raise_smem_limit((const void *)wfr_cols_kernel<T, S>, (int)G::SMEM));
    const Taps<T, S> gA = make_taps<T, S>(P.gy, P.sy, P.inv_norm);
    dim3 grid(P.pitch / 32, (P.H + G::TY - 1) / G::TY, P.nfx);
    wfr_cols_kernel<T, S><<<grid, G::THREADS, G::SMEM, s>>>(P.tmR, (const C2<T> *)P.d_ex, (const C2<T> *)P.d_ey,
                                                           P.nfy, P.W, P.H, P.pitch, gA, (T *)wb.pabs, wb.pk,
                                                           (T *)wb.pph, P.d_err);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

template <typename T>
static int enqueue_wfr_t(WffPlan &P, const WfrBuffers &wb, cudaStream_t s, const void *d_f, const glsu_wfr_results &z)
{
    GLSU_TRY(P.enqueue_rows(s, d_f));
    int rc;
    switch (P.syi) {
    case 12: rc = launch_wfr_cols<T, 12>(P, wb, s); break;
    case 20: rc = launch_wfr_cols<T, 20>(P, wb, s); break;
    case 30: rc = launch_wfr_cols<T, 30>(P, wb, s); break;
    case 45: rc = launch_wfr_cols<T, 45>(P, wb, s); break;
    default: rc = launch_wfr_cols<T, 60>(P, wb, s); break;
    }
    GLSU_TRY(rc);
    const int grid = std::min(P.H, 152 * 8);
    wfr_reduce_kernel<T><<<grid, 256, 0, s>>>((const T *)wb.pabs, wb.pk, (const T *)wb.pph, P.nfx, P.H, P.W,
                                              P.p.wxl, P.p.wxi, P.p.wyl, P.p.wyi, (T *)z.r, (T *)z.wx, (T *)z.wy,
                                              (T *)z.phase);
    WfrCurvTaps tp;
    tp.sx = P.sx;
    tp.sy = P.sy;
    double sxx = 0, sgx = 0, syy = 0, sgy = 0;
    for (int n = -P.sx; n <= P.sx; n++) {
        tp.gx[n + P.sx] = P.gx[n + P.sx];
        sxx += (double)n * n * P.gx[n + P.sx];
        sgx += P.gx[n + P.sx];
    }
    for (int m = -P.sy; m <= P.sy; m++) {
        tp.gy[m + P.sy] = P.gy[m + P.sy];
        syy += (double)m * m * P.gy[m + P.sy];
        sgy += P.gy[m + P.sy];
    }
    wfr_curv_rows_kernel<T><<<grid, 256, 0, s>>>((const T *)z.wx, (const T *)z.wy, P.H, P.W, tp, (T *)wb.A,
                                                 (T *)wb.B);
    wfr_final_kernel<T><<<grid, 256, 0, s>>>((const T *)wb.A, (const T *)wb.B, P.H, P.W, tp, sxx * sgy, syy * sgx,
                                             P.p.sigma_x, P.p.sigma_y, (const T *)z.r, (const T *)z.phase, (T *)z.cxx,
                                             (T *)z.cyy, (T *)z.phase_comp, (T *)z.b);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

int enqueue_wfr(WffPlan &P, const WfrBuffers &wb, cudaStream_t s, const void *d_f, const glsu_wfr_results &z)
{
    if (P.prec == GLSU_F32) return enqueue_wfr_t<float>(P, wb, s, d_f, z);
    return enqueue_wfr_t<double>(P, wb, s, d_f, z);
}

int WfrBuffers::alloc(const WffPlan &P)
{
    const size_t N = (size_t)P.W * P.H, es = P.prec == GLSU_F32 ? 4 : 8;
    if (cudaMalloc(&pabs, es * N * P.nfx) != cudaSuccess || cudaMalloc((void **)&pk, 4 * N * P.nfx) != cudaSuccess ||
        cudaMalloc(&pph, es * N * P.nfx) != cudaSuccess || cudaMalloc(&A, es * N) != cudaSuccess ||
        cudaMalloc(&B, es * N) != cudaSuccess)
        return fail(GLSU_ERR_ALLOC, "cudaMalloc of the WFR2 scratch failed");
    return GLSU_OK;
}

void WfrBuffers::release()
{
    cudaFree(pabs);
    cudaFree(pk);
    cudaFree(pph);
    cudaFree(A);
    cudaFree(B);
    pabs = pph = A = B = nullptr;
    pk = nullptr;
}

}  // namespace glsu
