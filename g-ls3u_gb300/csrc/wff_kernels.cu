// wff_kernels.cu -- WFF2 frequency sweep on sm_103a.
//
// The reference (WFT/WFT2_CPU.cpp:190-390, WFT/WFT2_CUDAf.cu:1016-1173)
// computes, for every frequency (wx, wy) on the grid,
//     sf  = f (*) w            w(y,x) = g(y,x) exp(j(wx x + wy y)), g the
//                              truncated, L2-normalised Gaussian window
//     sf  = sf .* (|sf| >= thr)
//     out += sf (*) w
// and scales out by wxi*wyi/(4 pi^2).  The reference evaluates each "(*)"
// as a cyclic convolution on an FFT-padded plane; the padding makes it a
// plain linear convolution with zero boundary, which is what is computed
// here, directly, with the same truncated window.
//
// Demodulation identity: (h (*) w)(n) = e^{j xi.n} ((h e^{-j xi.}) (*) g)(n).
// The window g is real and separable, and |sf| does not see the outer
// phase, so per frequency:
//     u   = (f e^{-j xi.}) (*) g        (real separable Gaussian filter)
//     out += e^{j xi.n} ((u .* [|u| >= thr]) (*) g)
// The x-filter of the first convolution does not depend on wy and the
// x-filter of the second commutes with the sum over wy, so a frame costs
// nfx row passes + nfx*nfy*2 column passes + nfx row passes:
//   A  wff_rows_demod   R_i = (f e^{-j wx_i x}) (*)_x gx           (nfx planes)
//   B  wff_cols         for each wy_k: u = (R_i e^{-j wy_k y}) (*)_y gy/N,
//                       threshold, c = t (*)_y gy, C_i += e^{j wy_k y} c
//   C  wff_rows_final   out = sum_i e^{j wx_i x} (C_i (*)_x gx) * scale/N
// Kernel B holds the column tile of R_i in shared memory (loaded by TMA,
// zero-filled outside the image) for all nfy frequencies.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "glsu_internal.cuh"
#include "wff_common.cuh"
#include "ptx_sm103.cuh"

namespace glsu {

// ---------------------------------------------------------------------------
// geometry
// ---------------------------------------------------------------------------
constexpr int kRowTileRows = 32;   // rows per CTA of the row kernels (one per lane)
constexpr int kRowTileCols = 128;  // output columns per CTA (8 warps x 16)
constexpr int kRowK = 16;          // output columns per thread
constexpr int kPitchAlign = 128;   // row pitch of the internal planes

template <typename T, int S> struct RowGeom {
    static constexpr int IN_W = kRowTileCols + 2 * S;
    static constexpr int IN_STRIDE = IN_W | 1;  // odd: lane-per-row access is conflict-free
    static constexpr int OUT_STRIDE = kRowTileCols + 1;
    static constexpr size_t SMEM =
        sizeof(C2<T>) * (size_t)(kRowTileRows * IN_STRIDE + kRowTileRows * OUT_STRIDE);
};

template <typename T, int S> struct ColGeom {
    // 8 warps; FP32 tiles of 128 output rows (the first filter recomputes a
    // 2S-row halo, 1.47x at S = 30).  A 16-warp, 256-row variant cut that to
    // 1.23x but ran no faster: at 128 registers per thread it spills.
    static constexpr int WARPS = 8;
    static constexpr int THREADS = 32 * WARPS;
    static constexpr int TY = (sizeof(T) == 4) ? 128 : (S <= 30 ? 64 : 32);  // output rows per CTA
    static constexpr int ROWS_U = TY + 2 * S;                                // rows of u / t
    static constexpr int KU = (ROWS_U + WARPS - 1) / WARPS;                  // u rows per warp
    static constexpr int KC = TY / WARPS;                                    // output rows per warp
    static constexpr int ROWS_R = TY + 4 * S;                                // rows of R needed
    static constexpr int BOX = (sizeof(T) == 4) ? 64 : 16;                   // rows per TMA box
    static constexpr int NBOX = (ROWS_R + BOX - 1) / BOX;
    static constexpr int RT = (NBOX * BOX > WARPS * KU + 2 * S) ? NBOX * BOX : WARPS * KU + 2 * S;
    static constexpr int TT = WARPS * KU;
    static constexpr int FPC = (int)(sizeof(C2<T>) / 4);  // floats per complex element
    static constexpr uint32_t TX_BYTES = (uint32_t)(NBOX * BOX * 32 * sizeof(C2<T>));
    static constexpr size_t SMEM = sizeof(C2<T>) * (size_t)(RT + TT) * 32 + 16;
    static_assert(SMEM <= 227 * 1024, "column tile exceeds shared memory");
};

// ---------------------------------------------------------------------------
// A: row pass with demodulation
// ---------------------------------------------------------------------------
template <typename T, int S>
__global__ void __launch_bounds__(256) wff_rows_demod_kernel(const C2<T> *__restrict__ f, int W, int H,
                                                             int pitch, const C2<T> *__restrict__ ex, int nfx,
                                                             C2<T> *__restrict__ R, Taps<T, S> gx, TileMask tm)
{
    using G = RowGeom<T, S>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<T> *ft = reinterpret_cast<C2<T> *>(smem_raw);
    C2<T> *ot = ft + kRowTileRows * G::IN_STRIDE;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int x0 = blockIdx.x * kRowTileCols, y0 = blockIdx.y * kRowTileRows;
    if (tm.flags && !tm.any(y0, y0 + kRowTileRows, x0, x0 + kRowTileCols)) return;

    for (int e = tid; e < kRowTileRows * G::IN_W; e += 256) {
        const int r = e / G::IN_W, c = e - r * G::IN_W;
        const int gy = y0 + r, gxx = x0 - S + c;
        C2<T> v = mk<T>(0, 0);
        if (gy < H && gxx >= 0 && gxx < W) v = f[(size_t)gy * W + gxx];
        ft[r * G::IN_STRIDE + c] = v;
    }
    __syncthreads();

    const size_t exs = (size_t)pitch + 2 * kPhasorPad;
    const size_t plane = (size_t)H * pitch;
    const C2<T> *row = ft + lane * G::IN_STRIDE + w * kRowK;
    for (int i = 0; i < nfx; i++) {
        const C2<T> *exi = ex + i * exs + kPhasorPad + (x0 - S + w * kRowK);
        T ar[kRowK], ai[kRowK];
#pragma unroll
        for (int k = 0; k < kRowK; k++) {
            ar[k] = 0;
            ai[k] = 0;
        }
#pragma unroll
        for (int j = 0; j < kRowK + 2 * S; j++) {
            const C2<T> v = row[j];
            const C2<T> p = __ldg(exi + j);
            const T dx = v.x * p.x - v.y * p.y;
            const T dy = v.x * p.y + v.y * p.x;
#pragma unroll
            for (int k = 0; k < kRowK; k++) {
                const int m = j - k;
                if (m >= 0 && m <= 2 * S) {
                    ar[k] = fma(gx.g[m], dx, ar[k]);
                    ai[k] = fma(gx.g[m], dy, ai[k]);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kRowK; k++) {
            const int gxx = x0 + w * kRowK + k;
            ot[lane * G::OUT_STRIDE + w * kRowK + k] = (gxx < W) ? mk<T>(ar[k], ai[k]) : mk<T>(0, 0);
        }
        __syncthreads();
        C2<T> *Ri = R + i * plane;
        for (int e = tid; e < kRowTileRows * kRowTileCols; e += 256) {
            const int r = e / kRowTileCols, c = e - r * kRowTileCols;
            const int gy = y0 + r, gxx = x0 + c;
            if (gy < H && gxx < pitch) Ri[(size_t)gy * pitch + gxx] = ot[r * G::OUT_STRIDE + c];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// B: column sweep over all wy for one wx and one 32-column tile
// ---------------------------------------------------------------------------
// One 32-column x TY-row tile of the sweep for wx index i; the mbarrier
// phase of this tile's TMA load is `parity`.  False when the load timed out.
template <typename T, int S>
__device__ __forceinline__ bool cols_tile(const CUtensorMap &tmR, C2<T> *__restrict__ Cout,
                                          const C2<T> *__restrict__ ey, int nfy, int H, int pitch, T thr, T thr2,
                                          const Taps<T, S> &gA, const Taps<T, S> &gB, int *__restrict__ err,
                                          C2<T> *Rt, C2<T> *tt, uint64_t *bar, uint32_t parity, int x0, int y0,
                                          int i)
{
    using G = ColGeom<T, S>;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const size_t eys = (size_t)H + 2 * kPhasorPad;
    if (tid == 0) {
        mbar_expect_tx(bar, G::TX_BYTES);
#pragma unroll 1
        for (int b = 0; b < G::NBOX; b++)
            tma_load_3d(Rt + b * G::BOX * 32, &tmR, bar, x0 * G::FPC, y0 - 2 * S + b * G::BOX, i);
    }
    for (int e = G::NBOX * G::BOX * 32 + tid; e < G::RT * 32; e += G::THREADS) Rt[e] = mk<T>(0, 0);
    const bool late = !mbar_wait_bounded(bar, parity);
    if (__syncthreads_or(late)) {
        if (tid == 0) {
            atomicExch(err, GLSU_ERR_TIMEOUT);
            mbar_wait_bounded(bar, parity);  // let copies still in flight land before exit
        }
        __syncthreads();
        return false;
    }

    T cr_acc[G::KC], ci_acc[G::KC];
#pragma unroll
    for (int k = 0; k < G::KC; k++) {
        cr_acc[k] = 0;
        ci_acc[k] = 0;
    }

    for (int k = 0; k < nfy; k++) {
        const C2<T> *eyk = ey + k * eys + kPhasorPad;
        // ---- pass 1: u over rows y0-S .. y0+TY+S-1, threshold into tt ----
        {
            const int q0 = w * G::KU;
            C2<T> a[G::KU];
#pragma unroll
            for (int kk = 0; kk < G::KU; kk++) a[kk] = mk<T>(0, 0);
#pragma unroll
            for (int j = 0; j < G::KU + 2 * S; j++) {
                const int q = q0 + j;
                const C2<T> r = Rt[q * 32 + lane];
                int gr = y0 - 2 * S + q;
                gr = min(max(gr, -kPhasorPad), H - 1 + kPhasorPad);
                const C2<T> p = __ldg(eyk + gr);
                const C2<T> d = mk<T>(r.x * p.x - r.y * p.y, r.x * p.y + r.y * p.x);
#pragma unroll
                for (int kk = 0; kk < G::KU; kk++) {
                    const int m = j - kk;
                    if (m >= 0 && m <= 2 * S) cfma(a[kk], gA.g[m], d);
                }
            }
#pragma unroll
            for (int kk = 0; kk < G::KU; kk++) {
                const int lr = q0 + kk;
                if (lr < G::ROWS_U) {
                    const int gr = y0 - S + lr;
                    bool keep = (gr >= 0) && (gr < H);
                    if (sizeof(T) == 8)
                        keep = keep && (sqrt(a[kk].x * a[kk].x + a[kk].y * a[kk].y) >= thr);
                    else
                        keep = keep && (a[kk].x * a[kk].x + a[kk].y * a[kk].y >= thr2);
                    tt[lr * 32 + lane] = keep ? a[kk] : mk<T>(0, 0);
                }
            }
        }
        __syncthreads();
        // ---- pass 2: c = t (*)_y gy, C += e^{+j wy y} c ----
        {
            const int o0 = w * G::KC;
            C2<T> c[G::KC];
#pragma unroll
            for (int kk = 0; kk < G::KC; kk++) c[kk] = mk<T>(0, 0);
#pragma unroll
            for (int j = 0; j < G::KC + 2 * S; j++) {
                const C2<T> t = tt[(o0 + j) * 32 + lane];
#pragma unroll
                for (int kk = 0; kk < G::KC; kk++) {
                    const int m = j - kk;
                    if (m >= 0 && m <= 2 * S) cfma(c[kk], gB.g[m], t);
                }
            }
#pragma unroll
            for (int kk = 0; kk < G::KC; kk++) {
                const int gr = min(y0 + o0 + kk, H - 1);
                const C2<T> p = __ldg(eyk + gr);  // e^{-j wy y}; multiply by its conjugate
                cr_acc[kk] += p.x * c[kk].x + p.y * c[kk].y;
                ci_acc[kk] += p.x * c[kk].y - p.y * c[kk].x;
            }
        }
        __syncthreads();
    }

    C2<T> *Ci = Cout + (size_t)i * H * pitch;
#pragma unroll
    for (int kk = 0; kk < G::KC; kk++) {
        const int gr = y0 + w * G::KC + kk;
        if (gr < H) Ci[(size_t)gr * pitch + x0 + lane] = mk<T>(cr_acc[kk], ci_acc[kk]);
    }
    return true;
}

template <typename T, int S>
__global__ void __launch_bounds__(ColGeom<T, S>::THREADS, 1)
    wff_cols_kernel(const __grid_constant__ CUtensorMap tmR, C2<T> *__restrict__ Cout,
                    const C2<T> *__restrict__ ey, int nfy, int H, int pitch, const T *__restrict__ thr_ptr,
                    Taps<T, S> gA, Taps<T, S> gB, int *__restrict__ err)
{
    using G = ColGeom<T, S>;
    extern __shared__ __align__(1024) unsigned char smem_cols[];
    C2<T> *Rt = reinterpret_cast<C2<T> *>(smem_cols);
    C2<T> *tt = Rt + G::RT * 32;
    uint64_t *bar = reinterpret_cast<uint64_t *>(tt + G::TT * 32);
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const T thr = *thr_ptr;
    cols_tile<T, S>(tmR, Cout, ey, nfy, H, pitch, thr, thr * thr, gA, gB, err, Rt, tt, bar, 0,
                    blockIdx.x * 32, blockIdx.y * G::TY, blockIdx.z);
}

// Tile-masked runs: the CTAs of each wx walk the device list of needed tiles.
template <typename T, int S>
__global__ void __launch_bounds__(ColGeom<T, S>::THREADS, 1)
    wff_cols_list_kernel(const __grid_constant__ CUtensorMap tmR, C2<T> *__restrict__ Cout,
                         const C2<T> *__restrict__ ey, int nfy, int H, int pitch, const T *__restrict__ thr_ptr,
                         Taps<T, S> gA, Taps<T, S> gB, int *__restrict__ err, const int2 *__restrict__ list,
                         const int *__restrict__ list_count)
{
    using G = ColGeom<T, S>;
    extern __shared__ __align__(1024) unsigned char smem_cols[];
    C2<T> *Rt = reinterpret_cast<C2<T> *>(smem_cols);
    C2<T> *tt = Rt + G::RT * 32;
    uint64_t *bar = reinterpret_cast<uint64_t *>(tt + G::TT * 32);
    const int nitems = *list_count;
    if ((int)blockIdx.x >= nitems) return;  // uniform, before any barrier or copy
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const T thr = *thr_ptr;
    uint32_t iter = 0;
    for (int item = blockIdx.x; item < nitems; item += gridDim.x, iter++) {
        const int2 tile = list[item];
        __syncthreads();  // the previous item is done with Rt and tt
        if (!cols_tile<T, S>(tmR, Cout, ey, nfy, H, pitch, thr, thr * thr, gA, gB, err, Rt, tt, bar, iter & 1,
                             tile.x * 32, tile.y * G::TY, blockIdx.z))
            return;
    }
}

// Tiles (bx, by) of ty_rows x tx_cols outputs of a column sweep whose
// outputs, grown by the mask's margins, meet a flagged tile, compacted in
// index order (one block; deterministic).
__global__ void __launch_bounds__(1024) wff_mask_list_kernel(TileMask m, int ncx, int ncy, int ty_rows, int tx_cols,
                                                             int2 *__restrict__ list, int *__restrict__ count)
{
    __shared__ int warp_sums[32];
    __shared__ int base;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    const int n = ncx * ncy;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c0 = 0; c0 < n; c0 += 1024) {
        const int e = c0 + threadIdx.x;
        int need = 0, bx = 0, by = 0;
        if (e < n) {
            by = e / ncx;
            bx = e - by * ncx;
            need = m.any(by * ty_rows, by * ty_rows + ty_rows, bx * tx_cols, bx * tx_cols + tx_cols) ? 1 : 0;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, need);
        if (lane == 0) warp_sums[w] = __popc(bal);
        __syncthreads();
        int before = 0;
        for (int q = 0; q < w; q++) before += warp_sums[q];
        if (need) list[base + before + __popc(bal & ((1u << lane) - 1u))] = make_int2(bx, by);
        __syncthreads();
        if (threadIdx.x == 0) {
            int tot = 0;
            for (int q = 0; q < 32; q++) tot += warp_sums[q];
            base += tot;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = base;
}

// ---------------------------------------------------------------------------
// C: final row pass, modulation, sum over wx (+ optional DPRA phase update)
// ---------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T wrap_atan2(T a);
template <> __device__ __forceinline__ float wrap_atan2<float>(float a)
{
    float s, c;
    sincosf(a, &s, &c);
    return atan2f(s, c);
}
template <> __device__ __forceinline__ double wrap_atan2<double>(double a)
{
    double s, c;
    sincos(a, &s, &c);
    return atan2(s, c);
}

template <typename T, int S, int MODE>
__global__ void __launch_bounds__(256) wff_rows_final_kernel(const C2<T> *__restrict__ Cin, int W, int H,
                                                             int pitch, const C2<T> *__restrict__ ex, int nfx,
                                                             Taps<T, S> gx, C2<T> *__restrict__ out,
                                                             const T *__restrict__ phiref,
                                                             const T *__restrict__ dphiref,
                                                             T *__restrict__ phicurr, T *__restrict__ dphi,
                                                             TileMask tm)
{
    using G = RowGeom<T, S>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<T> *ft = reinterpret_cast<C2<T> *>(smem_raw);
    C2<T> *ot = ft + kRowTileRows * G::IN_STRIDE;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int x0 = blockIdx.x * kRowTileCols, y0 = blockIdx.y * kRowTileRows;
    if (tm.flags && !tm.any(y0, y0 + kRowTileRows, x0, x0 + kRowTileCols)) return;
    const size_t exs = (size_t)pitch + 2 * kPhasorPad;
    const size_t plane = (size_t)H * pitch;

    T orr[kRowK], oii[kRowK];
#pragma unroll
    for (int k = 0; k < kRowK; k++) {
        orr[k] = 0;
        oii[k] = 0;
    }
    const C2<T> *row = ft + lane * G::IN_STRIDE + w * kRowK;
    for (int i = 0; i < nfx; i++) {
        const C2<T> *Ci = Cin + i * plane;
        for (int e = tid; e < kRowTileRows * G::IN_W; e += 256) {
            const int r = e / G::IN_W, c = e - r * G::IN_W;
            const int gy = y0 + r, gxx = x0 - S + c;
            C2<T> v = mk<T>(0, 0);
            if (gy < H && gxx >= 0 && gxx < W) v = Ci[(size_t)gy * pitch + gxx];
            ft[r * G::IN_STRIDE + c] = v;
        }
        __syncthreads();
        T ar[kRowK], ai[kRowK];
#pragma unroll
        for (int k = 0; k < kRowK; k++) {
            ar[k] = 0;
            ai[k] = 0;
        }
#pragma unroll
        for (int j = 0; j < kRowK + 2 * S; j++) {
            const C2<T> v = row[j];
#pragma unroll
            for (int k = 0; k < kRowK; k++) {
                const int m = j - k;
                if (m >= 0 && m <= 2 * S) {
                    ar[k] = fma(gx.g[m], v.x, ar[k]);
                    ai[k] = fma(gx.g[m], v.y, ai[k]);
                }
            }
        }
        const C2<T> *exi = ex + i * exs + kPhasorPad + (x0 + w * kRowK);
#pragma unroll
        for (int k = 0; k < kRowK; k++) {
            const C2<T> p = __ldg(exi + k);  // e^{-j wx x}; multiply by its conjugate
            orr[k] += p.x * ar[k] + p.y * ai[k];
            oii[k] += p.x * ai[k] - p.y * ar[k];
        }
        __syncthreads();
    }

#pragma unroll
    for (int k = 0; k < kRowK; k++) ot[lane * G::OUT_STRIDE + w * kRowK + k] = mk<T>(orr[k], oii[k]);
    __syncthreads();
    for (int e = tid; e < kRowTileRows * kRowTileCols; e += 256) {
        const int r = e / kRowTileCols, c = e - r * kRowTileCols;
        const int gy = y0 + r, gxx = x0 + c;
        if (gy >= H || gxx >= W) continue;
        if (tm.flags && !tm.at(gy, gxx)) continue;
        const size_t id = (size_t)gy * W + gxx;
        const C2<T> v = ot[r * G::OUT_STRIDE + c];
        if (MODE == 0) {
            out[id] = v;
        } else {
            // DPRA update (DPRA/dpra_hybrid.cu:297-315, DPRA/dpra_cpu.cpp:243-249)
            const T t = atan2(v.y, v.x);
            const T pr = phiref[id];
            phicurr[id] = wrap_atan2<T>(t + pr);
            // MODE 2 leaves the wrapped change t for the spatial unwrapping,
            // which adds dphi_ref afterwards (MatLab/fp_ls3u.m:104)
            dphi[id] = (MODE == 1) ? dphiref[id] + t : t;
        }
    }
}

// ---------------------------------------------------------------------------
// automatic threshold: thr = 6 sqrt(mean|f|^2 / 3)  (WFT/WFT2_CPU.cpp:977-1005)
// ---------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(256) wff_thr_partial_kernel(const C2<T> *__restrict__ f, size_t n,
                                                              double *__restrict__ part)
{
    __shared__ double red[256];
    double acc = 0;
    for (size_t k = blockIdx.x * 256 + threadIdx.x; k < n; k += (size_t)gridDim.x * 256) {
        const C2<T> v = f[k];
        acc += (double)v.x * v.x + (double)v.y * v.y;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

template <typename T>
__global__ void wff_thr_final_kernel(const double *__restrict__ part, int nb, size_t n, T *__restrict__ thr)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0;
        for (int b = 0; b < nb; b++) s += part[b];
        *thr = (T)(6.0 * sqrt(s / (double)n / 3.0));
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int instantiated_half(int s)
{
    if (s < 0) return -1;
    if (s <= 12) return 12;
    if (s <= 20) return 20;
    if (s <= 30) return 30;
    if (s <= 45) return 45;
    if (s <= 60) return 60;
    return -1;
}

static int count_freq(double lo, double hi, double step, int prec)
{
    if (prec == GLSU_F32) {
        const float l = (float)lo, h = (float)hi, st = (float)step;
        const float v = (h - l) * (1.0f / st);
        return (int)v + 1;
    }
    return (int)((hi - lo) * (1.0 / step)) + 1;
}

int wff_count_public(double lo, double hi, double step, int prec) { return count_freq(lo, hi, step, prec); }

size_t WffPlan::plane_bytes() const
{
    return (size_t)H * pitch * (prec == GLSU_F32 ? sizeof(float2) : sizeof(double2));
}

int WffPlan::init(int precision, int width, int height, const glsu_wff_params &prm)
{
    if (precision != GLSU_F32 && precision != GLSU_F64) return fail(GLSU_ERR_INVALID, "precision must be F32 or F64");
    if (width < 1 || height < 1) return fail(GLSU_ERR_INVALID, "image size must be positive");
    if (!(prm.sigma_x > 0) || !(prm.sigma_y > 0)) return fail(GLSU_ERR_INVALID, "sigma must be positive");
    if (!(prm.wxi > 0) || !(prm.wyi > 0)) return fail(GLSU_ERR_INVALID, "frequency step must be positive");
    if (!(prm.wxh >= prm.wxl) || !(prm.wyh >= prm.wyl))
        return fail(GLSU_ERR_INVALID, "frequency upper bound below lower bound");
    prec = precision;
    W = width;
    H = height;
    p = prm;
    sx = (int)std::lround(3 * prm.sigma_x);
    sy = (int)std::lround(3 * prm.sigma_y);
    Wp = glsu_opt_fft_size(W + 2 * sx);
    Hp = glsu_opt_fft_size(H + 2 * sy);
    if (Wp < 0 || Hp < 0)
        return fail(GLSU_ERR_PADDING,
                    "FFT padding is out of range [4096]. Shrink the size of either the image or the Gaussian Window!");
    sxi = instantiated_half(sx);
    syi = instantiated_half(sy);
    if (sxi < 0 || syi < 0) return fail(GLSU_ERR_UNSUPPORTED, "window half-size round(3*sigma) above 60");
    nfx = count_freq(prm.wxl, prm.wxh, prm.wxi, prec);
    nfy = count_freq(prm.wyl, prm.wyh, prm.wyi, prec);
    if (nfx < 1 || nfy < 1 || nfx > 4096 || nfy > 4096) return fail(GLSU_ERR_INVALID, "bad frequency grid");
    pitch = (W + kPitchAlign - 1) / kPitchAlign * kPitchAlign;

    // taps (double on the host; cast per precision at launch)
    double sgx = 0, sgy = 0;
    for (int m = -sx; m <= sx; m++) {
        const double v = std::exp(-(double)(m * m) / 2 / prm.sigma_x / prm.sigma_x);
        gx[m + sx] = v;
        sgx += v * v;
    }
    for (int m = -sy; m <= sy; m++) {
        const double v = std::exp(-(double)(m * m) / 2 / prm.sigma_y / prm.sigma_y);
        gy[m + sy] = v;
        sgy += v * v;
    }
    inv_norm = 1.0 / std::sqrt(sgx * sgy);
    scale = 0.25 * (1.0 / (M_PI * M_PI)) * prm.wxi * prm.wyi;
    thr_ready = false;
    thr_host = prm.thr;
    return GLSU_OK;
}

int WffPlan::alloc_device()
{
    const size_t cs = prec == GLSU_F32 ? sizeof(float2) : sizeof(double2);
    const size_t exn = (size_t)nfx * (pitch + 2 * kPhasorPad), eyn = (size_t)nfy * (H + 2 * kPhasorPad);
    if (cudaMalloc(&d_ex, exn * cs) != cudaSuccess || cudaMalloc(&d_ey, eyn * cs) != cudaSuccess)
        return fail(GLSU_ERR_ALLOC, "cudaMalloc of phasor tables failed");
    if (!external_scratch) {
        if (cudaMalloc(&d_R, (size_t)nfx * plane_bytes()) != cudaSuccess ||
            cudaMalloc(&d_C, (size_t)nfx * plane_bytes()) != cudaSuccess)
            return fail(GLSU_ERR_ALLOC, "cudaMalloc of WFF2 planes failed");
        // defined contents: a tile-masked run reads planes it did not write
        GLSU_CUDA_TRY(cudaMemset(d_R, 0, (size_t)nfx * plane_bytes()));
        GLSU_CUDA_TRY(cudaMemset(d_C, 0, (size_t)nfx * plane_bytes()));
        if (cudaMalloc(&d_thr, sizeof(double)) != cudaSuccess ||
            cudaMalloc((void **)&d_part, sizeof(double) * kThrBlocks) != cudaSuccess ||
            cudaMalloc((void **)&d_err, sizeof(int)) != cudaSuccess)
            return fail(GLSU_ERR_ALLOC, "cudaMalloc failed");
        GLSU_CUDA_TRY(cudaMemset(d_err, 0, sizeof(int)));
    }
    return GLSU_OK;
}

int WffPlan::upload_tables(cudaStream_t s)
{
    const size_t exs = (size_t)pitch + 2 * kPhasorPad, eys = (size_t)H + 2 * kPhasorPad;
    std::vector<double> ex(2 * nfx * exs), ey(2 * nfy * eys);
    for (int i = 0; i < nfx; i++) {
        const double wx = p.wxl + (double)i * p.wxi;
        for (size_t t = 0; t < exs; t++) {
            const double x = (double)t - kPhasorPad;
            ex[2 * (i * exs + t)] = std::cos(wx * x);
            ex[2 * (i * exs + t) + 1] = -std::sin(wx * x);
        }
    }
    for (int k = 0; k < nfy; k++) {
        const double wy = p.wyl + (double)k * p.wyi;
        for (size_t t = 0; t < eys; t++) {
            const double y = (double)t - kPhasorPad;
            ey[2 * (k * eys + t)] = std::cos(wy * y);
            ey[2 * (k * eys + t) + 1] = -std::sin(wy * y);
        }
    }
    if (prec == GLSU_F32) {
        std::vector<float> exf(ex.begin(), ex.end()), eyf(ey.begin(), ey.end());
        GLSU_CUDA_TRY(cudaMemcpy(d_ex, exf.data(), exf.size() * sizeof(float), cudaMemcpyHostToDevice));
        GLSU_CUDA_TRY(cudaMemcpy(d_ey, eyf.data(), eyf.size() * sizeof(float), cudaMemcpyHostToDevice));
        if (p.thr >= 0) {
            const float t = (float)p.thr;
            GLSU_CUDA_TRY(cudaMemcpy(d_thr, &t, sizeof(float), cudaMemcpyHostToDevice));
        }
    } else {
        GLSU_CUDA_TRY(cudaMemcpy(d_ex, ex.data(), ex.size() * sizeof(double), cudaMemcpyHostToDevice));
        GLSU_CUDA_TRY(cudaMemcpy(d_ey, ey.data(), ey.size() * sizeof(double), cudaMemcpyHostToDevice));
        if (p.thr >= 0) GLSU_CUDA_TRY(cudaMemcpy(d_thr, &p.thr, sizeof(double), cudaMemcpyHostToDevice));
    }
    (void)s;
    return GLSU_OK;
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
    }
    return fn;
}

int WffPlan::make_tensor_map()
{
    auto enc = get_encode_fn();
    if (!enc) return fail(GLSU_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    const int fpc = prec == GLSU_F32 ? 2 : 4;
    const int box = prec == GLSU_F32 ? 64 : 16;
    cuuint64_t dims[3] = {(cuuint64_t)pitch * fpc, (cuuint64_t)H, (cuuint64_t)nfx};
    cuuint64_t strides[2] = {(cuuint64_t)pitch * fpc * 4, (cuuint64_t)H * pitch * fpc * 4};
    cuuint32_t boxd[3] = {(cuuint32_t)(32 * fpc), (cuuint32_t)box, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc(&tmR, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, d_R, dims, strides, boxd, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(GLSU_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    return GLSU_OK;
}

int WffPlan::alloc_tile_list()
{
    if (d_list) return GLSU_OK;
    // column tiles of the direct sweep are 32 columns x at least 32 rows;
    // column groups of the FFT sweep are 1 to 16 whole columns
    const size_t cap = std::max((size_t)(pitch / 32) * ((H + 31) / 32), (size_t)pitch);
    if (cudaMalloc((void **)&d_list, cap * sizeof(int2)) != cudaSuccess ||
        cudaMalloc((void **)&d_list_count, sizeof(int)) != cudaSuccess)
        return fail(GLSU_ERR_ALLOC, "cudaMalloc of the tile list failed");
    return GLSU_OK;
}

void WffPlan::release()
{
    release_colfft();
    cudaFree(d_ex);
    cudaFree(d_ey);
    cudaFree(d_list);
    cudaFree(d_list_count);
    d_ex = d_ey = nullptr;
    d_list = nullptr;
    d_list_count = nullptr;
    if (!external_scratch) {
        cudaFree(d_R);
        cudaFree(d_C);
        cudaFree(d_thr);
        cudaFree(d_part);
        cudaFree(d_err);
    }
    d_R = d_C = d_thr = nullptr;
    d_part = nullptr;
    d_err = nullptr;
}

int WffPlan::check_device_error(cudaStream_t s)
{
    int e = 0;
    GLSU_CUDA_TRY(cudaMemcpyAsync(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    GLSU_CUDA_TRY(cudaStreamSynchronize(s));
    if (e) {
        cudaMemsetAsync(d_err, 0, sizeof(int), s);
        return fail(e, "a bounded device-side wait timed out in the WFF2 column sweep");
    }
    return GLSU_OK;
}

// ---- launch dispatch ------------------------------------------------------
int launch_mask_list(const TileMask &m, int ncx, int ncy, int ty_rows, int tx_cols, int2 *list, int *count,
                     cudaStream_t s)
{
    wff_mask_list_kernel<<<1, 1024, 0, s>>>(m, ncx, ncy, ty_rows, tx_cols, list, count);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

static TileMask with_margins(TileMask m, int my, int mx)
{
    m.my = my;
    m.mx = mx;
    return m;
}

template <typename T, int S>
static int launch_rows_demod(const WffPlan &P, const void *d_f, cudaStream_t s)
{
    using G = RowGeom<T, S>;
    GLSU_TRY(raise_smem_limit((const void *)wff_rows_demod_kernel<T, S>, (int)G::SMEM));
    dim3 grid(P.pitch / kRowTileCols, (P.H + kRowTileRows - 1) / kRowTileRows);
    wff_rows_demod_kernel<T, S><<<grid, 256, G::SMEM, s>>>(
        (const C2<T> *)d_f, P.W, P.H, P.pitch, (const C2<T> *)P.d_ex, P.nfx, (C2<T> *)P.d_R,
        make_taps<T, S>(P.gx, P.sx, 1.0), with_margins(P.mask, 2 * P.sy, P.sx));
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

int WffPlan::enqueue_rows(cudaStream_t s, const void *d_f)
{
    if (mask.flags) return fail(GLSU_ERR_INVALID, "full-frame row pass with a tile mask set");
#define GLSU_ROWS(SS) \
    return prec == GLSU_F32 ? launch_rows_demod<float, SS>(*this, d_f, s) : launch_rows_demod<double, SS>(*this, d_f, s);
    switch (sxi) {
    case 12: GLSU_ROWS(12)
    case 20: GLSU_ROWS(20)
    case 30: GLSU_ROWS(30)
    case 45: GLSU_ROWS(45)
    default: GLSU_ROWS(60)
    }
#undef GLSU_ROWS
}

template <typename T, int S> static int launch_cols(const WffPlan &P, cudaStream_t s)
{
    using G = ColGeom<T, S>;
    GLSU_TRY(raise_smem_limit((const void *)wff_cols_kernel<T, S>, (int)G::SMEM));
    const int ncx = P.pitch / 32, ncy = (P.H + G::TY - 1) / G::TY;
    const Taps<T, S> gA = make_taps<T, S>(P.gy, P.sy, P.inv_norm), gB = make_taps<T, S>(P.gy, P.sy, 1.0);
    if (!P.mask.flags) {
        wff_cols_kernel<T, S><<<dim3(ncx, ncy, P.nfx), G::THREADS, G::SMEM, s>>>(
            P.tmR, (C2<T> *)P.d_C, (const C2<T> *)P.d_ey, P.nfy, P.H, P.pitch, (const T *)P.d_thr, gA, gB, P.d_err);
    } else {
        // tile-masked run: compact the needed column tiles on the device and
        // let a few CTAs per wx walk that list (an empty list costs one short
        // launch instead of a full grid of CTAs that exit at once)
        GLSU_TRY(raise_smem_limit((const void *)wff_cols_list_kernel<T, S>, (int)G::SMEM));
        if (!P.d_list) return fail(GLSU_ERR_INVALID, "tile-masked run without a tile list buffer");
        GLSU_TRY(launch_mask_list(with_margins(P.mask, 0, P.sx), ncx, ncy, G::TY, 32, P.d_list, P.d_list_count, s));
        const int per_wx = std::max(1, std::min(ncx * ncy, (2 * 152 + P.nfx - 1) / P.nfx));
        wff_cols_list_kernel<T, S><<<dim3(per_wx, 1, P.nfx), G::THREADS, G::SMEM, s>>>(
            P.tmR, (C2<T> *)P.d_C, (const C2<T> *)P.d_ey, P.nfy, P.H, P.pitch, (const T *)P.d_thr, gA, gB, P.d_err,
            P.d_list, P.d_list_count);
    }
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

template <typename T, int S, int MODE>
static int launch_final(const WffPlan &P, void *d_out, const void *phiref, const void *dphiref, void *phicurr,
                        void *dphi, cudaStream_t s)
{
    using G = RowGeom<T, S>;
    GLSU_TRY(raise_smem_limit((const void *)wff_rows_final_kernel<T, S, MODE>, (int)G::SMEM));
    dim3 grid(P.pitch / kRowTileCols, (P.H + kRowTileRows - 1) / kRowTileRows);
    wff_rows_final_kernel<T, S, MODE><<<grid, 256, G::SMEM, s>>>(
        (const C2<T> *)P.d_C, P.W, P.H, P.pitch, (const C2<T> *)P.d_ex, P.nfx,
        make_taps<T, S>(P.gx, P.sx, P.scale * P.inv_norm), (C2<T> *)d_out, (const T *)phiref, (const T *)dphiref,
        (T *)phicurr, (T *)dphi, with_margins(P.mask, 0, 0));
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

template <typename T> static int launch_cols_any(WffPlan &P, cudaStream_t s)
{
    if (sizeof(T) == 4 && P.use_colfft()) return launch_colfft(P, s);
    switch (P.syi) {
    case 12: return launch_cols<T, 12>(P, s);
    case 20: return launch_cols<T, 20>(P, s);
    case 30: return launch_cols<T, 30>(P, s);
    case 45: return launch_cols<T, 45>(P, s);
    default: return launch_cols<T, 60>(P, s);
    }
}

int launch_column_sweep(WffPlan &P, cudaStream_t s)
{
    return P.prec == GLSU_F32 ? launch_cols_any<float>(P, s) : launch_cols_any<double>(P, s);
}

template <typename T>
static int enqueue_t(WffPlan &P, cudaStream_t s, const void *d_f, void *d_out, int mode, const void *phiref,
                     const void *dphiref, void *phicurr, void *dphi, cudaEvent_t *ev)
{
    GLSU_TRY(P.ensure_threshold(s, d_f));
    if (ev) GLSU_CUDA_TRY(cudaEventRecord(ev[0], s));
    int rc = GLSU_OK;
    switch (P.sxi) {
    case 12: rc = launch_rows_demod<T, 12>(P, d_f, s); break;
    case 20: rc = launch_rows_demod<T, 20>(P, d_f, s); break;
    case 30: rc = launch_rows_demod<T, 30>(P, d_f, s); break;
    case 45: rc = launch_rows_demod<T, 45>(P, d_f, s); break;
    default: rc = launch_rows_demod<T, 60>(P, d_f, s); break;
    }
    if (rc) return rc;
    if (ev) GLSU_CUDA_TRY(cudaEventRecord(ev[1], s));
    rc = launch_cols_any<T>(P, s);
    if (rc) return rc;
    if (ev) GLSU_CUDA_TRY(cudaEventRecord(ev[2], s));
#define GLSU_FINAL(SS)                                                                              \
    rc = mode == 0   ? launch_final<T, SS, 0>(P, d_out, phiref, dphiref, phicurr, dphi, s)          \
         : mode == 1 ? launch_final<T, SS, 1>(P, d_out, phiref, dphiref, phicurr, dphi, s)          \
                     : launch_final<T, SS, 2>(P, d_out, phiref, dphiref, phicurr, dphi, s);
    switch (P.sxi) {
    case 12: GLSU_FINAL(12) break;
    case 20: GLSU_FINAL(20) break;
    case 30: GLSU_FINAL(30) break;
    case 45: GLSU_FINAL(45) break;
    default: GLSU_FINAL(60) break;
    }
#undef GLSU_FINAL
    if (rc) return rc;
    if (ev) GLSU_CUDA_TRY(cudaEventRecord(ev[3], s));
    return GLSU_OK;
}

// The same three stages one at a time (the batched form interleaves them
// across sequences): threshold + row pass, column sweep, final row pass.
template <typename T> static int enqueue_pre_t(WffPlan &P, cudaStream_t s, const void *d_f)
{
    GLSU_TRY(P.ensure_threshold(s, d_f));
    switch (P.sxi) {
    case 12: return launch_rows_demod<T, 12>(P, d_f, s);
    case 20: return launch_rows_demod<T, 20>(P, d_f, s);
    case 30: return launch_rows_demod<T, 30>(P, d_f, s);
    case 45: return launch_rows_demod<T, 45>(P, d_f, s);
    default: return launch_rows_demod<T, 60>(P, d_f, s);
    }
}

#define GLSU_FINAL(SS)                                                                              \
    rc = mode == 0   ? launch_final<T, SS, 0>(P, d_out, phiref, dphiref, phicurr, dphi, s)          \
         : mode == 1 ? launch_final<T, SS, 1>(P, d_out, phiref, dphiref, phicurr, dphi, s)          \
                     : launch_final<T, SS, 2>(P, d_out, phiref, dphiref, phicurr, dphi, s);
template <typename T>
static int enqueue_final_t(WffPlan &P, cudaStream_t s, void *d_out, int mode, const void *phiref,
                           const void *dphiref, void *phicurr, void *dphi)
{
    int rc = GLSU_OK;
    switch (P.sxi) {
    case 12: GLSU_FINAL(12) break;
    case 20: GLSU_FINAL(20) break;
    case 30: GLSU_FINAL(30) break;
    case 45: GLSU_FINAL(45) break;
    default: GLSU_FINAL(60) break;
    }
    return rc;
}
#undef GLSU_FINAL

int WffPlan::enqueue_pre(cudaStream_t s, const void *d_f)
{
    if (mask.flags) return fail(GLSU_ERR_INVALID, "staged WFF2 with a tile mask set");
    return prec == GLSU_F32 ? enqueue_pre_t<float>(*this, s, d_f) : enqueue_pre_t<double>(*this, s, d_f);
}

int WffPlan::enqueue_final(cudaStream_t s, void *d_out, int final_mode, const void *phi_ref, const void *dphi_ref,
                           void *phi_curr, void *dphi)
{
    return prec == GLSU_F32 ? enqueue_final_t<float>(*this, s, d_out, final_mode, phi_ref, dphi_ref, phi_curr, dphi)
                            : enqueue_final_t<double>(*this, s, d_out, final_mode, phi_ref, dphi_ref, phi_curr, dphi);
}

int WffPlan::ensure_threshold(cudaStream_t s, const void *d_f)
{
    if (p.thr >= 0 || thr_ready) return GLSU_OK;
    const size_t n = (size_t)W * H;
    if (prec == GLSU_F32) {
        wff_thr_partial_kernel<float><<<kThrBlocks, 256, 0, s>>>((const float2 *)d_f, n, d_part);
        wff_thr_final_kernel<float><<<1, 32, 0, s>>>(d_part, kThrBlocks, n, (float *)d_thr);
    } else {
        wff_thr_partial_kernel<double><<<kThrBlocks, 256, 0, s>>>((const double2 *)d_f, n, d_part);
        wff_thr_final_kernel<double><<<1, 32, 0, s>>>(d_part, kThrBlocks, n, (double *)d_thr);
    }
    GLSU_CUDA_TRY(cudaGetLastError());
    thr_ready = true;
    return GLSU_OK;
}

int WffPlan::enqueue(cudaStream_t s, const void *d_f, void *d_out, int final_mode, const void *phi_ref,
                     const void *dphi_ref, void *phi_curr, void *dphi, cudaEvent_t *stage_ev)
{
    if (prec == GLSU_F32)
        return enqueue_t<float>(*this, s, d_f, d_out, final_mode, phi_ref, dphi_ref, phi_curr, dphi, stage_ev);
    return enqueue_t<double>(*this, s, d_f, d_out, final_mode, phi_ref, dphi_ref, phi_curr, dphi, stage_ev);
}

}  // namespace glsu
