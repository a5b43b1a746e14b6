// wff_probe.cu -- exact WFF2 on sparse patches: the check on the surrogate.
//
// For each tile of the frame, one P x P patch (position hashed from a seed
// and the tile index) gets the exact FP32 WFF2 output, computed by the same
// separable, demodulated formulation as the full-frame kernels (rows demod,
// column sweep with threshold, final rows; WFT/WFT2_CPU.cpp:190-390):
// one CTA per (tile, wx, part of the wy range), holding in shared memory
//   R  the row-filtered, demodulated input over rows py-2sy .. py+P+2sy-1
//      and columns px-sx .. px+P+sx-1 (zero outside the image, the crop),
//   U  the thresholded first column filter over rows py-sy .. py+P+sy-1,
//   C  the second column filter summed over wy on rows py .. py+P-1,
// then the final row filter on the P x P patch.  The per-wx partials are
// summed in a fixed order by the residual kernel, which compares the patch
// with the surrogate's output and flags the tile.
#include <algorithm>
#include <cmath>

#include "glsu_internal.cuh"

namespace glsu {

template <typename T, int S> struct PTaps {
    T g[2 * S + 1];
};

// Geometry of the probe for an instantiated window half-size S: the patch P
// is chosen so that P + 2S fills whole 32-lane column groups (lane = column).
template <int S> struct ProbeGeom {
    static constexpr int P = S <= 20 ? 8 : 4;
    static constexpr int RX = P + 2 * S;      // columns of R, U, C
    static constexpr int NCG = (RX + 31) / 32;
    static constexpr int RXP = NCG * 32;
    static constexpr int NRG = 4;              // warps along the rows
    static constexpr int THREADS = NCG * NRG * 32;
    static constexpr int UY = P + 2 * S;       // rows of U
    static constexpr int KU = (UY + NRG - 1) / NRG;
    static constexpr int UYP = NRG * KU;
    static constexpr int RYP = UYP + 2 * S;    // rows of R (>= P + 4S)
    static constexpr int CPT = (P + NRG - 1) / NRG;  // C rows per thread
    static constexpr size_t R_ELEMS = (size_t)RYP * RXP;  // one (tile, wx) block of R
    static constexpr size_t SMEM = sizeof(float2) * (R_ELEMS + (size_t)UYP * RXP + RYP);
    // row pass: a thread takes 16 adjacent columns of one row, 64 rows per chunk
    static constexpr int SEG = 16;
    static constexpr int NSEG = RXP / SEG;
    static constexpr int CR = 64;
    static constexpr int RTHREADS = NSEG * CR;
    static constexpr int FX = RXP + 2 * S;     // staged input columns
    static constexpr int FXS = FX | 1;         // odd row stride (float2): a warp's rows hit distinct bank pairs
    static constexpr size_t RSMEM = sizeof(float2) * ((size_t)CR * FXS + FX);
};

int probe_patch_for_half(int s_inst) { return s_inst <= 20 ? 8 : 4; }

size_t probe_rows_elems(int s_inst)
{
    switch (s_inst) {
    case 12: return ProbeGeom<12>::R_ELEMS;
    case 20: return ProbeGeom<20>::R_ELEMS;
    case 30: return ProbeGeom<30>::R_ELEMS;
    default: return ProbeGeom<45>::R_ELEMS;
    }
}

struct ProbeArgs {
    const float2 *f, *ex, *ey;
    const float *thr;
    int W, H, pitch, nfx, nfy, P;
    int tile, ntx, nty, nsplit;
    uint32_t seed;
    float2 *partial;  // [ntiles][nfx * nsplit][P*P]
    int2 *sites;
    float2 *rows;     // [ntiles][nfx][RYP][RXP]: R of each (tile, wx)
    const uint32_t *seed_dev;  // not null: the seed is read here (a frame counter on the device)
};

__device__ __forceinline__ uint32_t hash32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ int2 probe_site(const ProbeArgs &a, int t)
{
    const int ty = t / a.ntx, tx = t - ty * a.ntx;
    const int y0 = ty * a.tile, x0 = tx * a.tile;
    const int th = min(a.tile, a.H - y0), tw = min(a.tile, a.W - x0);
    const uint32_t h1 = hash32(a.seed * 0x9E3779B9u + (uint32_t)t * 0x85EBCA6Bu + 0x27D4EB2Fu);
    const uint32_t h2 = hash32(h1 ^ 0x165667B1u);
    return make_int2(y0 + (int)(h1 % (uint32_t)max(1, th - a.P + 1)), x0 + (int)(h2 % (uint32_t)max(1, tw - a.P + 1)));
}

// Row pass, one CTA per (tile, wx, chunk of 64 rows): R = the rows
// py-2S .. py-2S+RYP-1, demodulated by e^{-j wx x} and filtered along x, for
// the columns px-S .. px-S+RXP-1 (zero outside the image and beyond RX).  A
// thread takes 16 adjacent output columns of one row from 16+2S staged
// inputs, summing the taps in ascending order for each output.  Up to half
// size 30 the registers are capped for two CTAs per SM: the pass is latency
// bound, and the second CTA takes it from 49 to about 39 us at 1024^2 (a few
// bytes of spills); at half size 45 the cap would spill heavily.
template <int S>
__global__ void __launch_bounds__(ProbeGeom<S>::RTHREADS, (S <= 30 ? 2 : 1)) wff_probe_rows_kernel(ProbeArgs a, PTaps<float, S> gxr)
{
    using G = ProbeGeom<S>;
    constexpr int RX = G::RX, RXP = G::RXP, RYP = G::RYP, FX = G::FX, FXS = G::FXS, CR = G::CR, SEG = G::SEG;
    extern __shared__ __align__(16) float2 psm[];
    float2 *fs = psm;            // [CR][FXS] demodulated input rows
    float2 *es = fs + CR * FXS;  // [FX] e^{-j wx x}
    const int t = blockIdx.x, i = blockIdx.y, tid = threadIdx.x;
    const int rl = tid % CR, seg = tid / CR;
    if (a.seed_dev) a.seed = *a.seed_dev;
    const int2 site = probe_site(a, t);
    const int py = site.x, px = site.y;
    const float2 *exi = a.ex + (size_t)i * (a.pitch + 2 * kPhasorPad) + kPhasorPad;
    float2 *Rg = a.rows + ((size_t)t * gridDim.y + i) * G::R_ELEMS;
    for (int e = tid; e < FX; e += G::RTHREADS) es[e] = exi[px - 2 * S + e];
    {
        const int r0 = blockIdx.z * CR;
        __syncthreads();  // es is written
        for (int e = tid; e < CR * FX; e += G::RTHREADS) {
            const int rr = e / FX, c = e - rr * FX;
            const int y = py - 2 * S + r0 + rr, x = px - 2 * S + c;
            float2 v = make_float2(0.f, 0.f);
            if (r0 + rr < RYP && y >= 0 && y < a.H && x >= 0 && x < a.W) v = a.f[(size_t)y * a.W + x];
            const float2 p = es[c];
            fs[rr * FXS + c] = make_float2(v.x * p.x - v.y * p.y, v.x * p.y + v.y * p.x);
        }
        __syncthreads();
        float2 acc[SEG];
#pragma unroll
        for (int q = 0; q < SEG; q++) acc[q] = make_float2(0.f, 0.f);
        const float2 *row = fs + rl * FXS + seg * SEG;
#pragma unroll
        for (int j = 0; j < SEG + 2 * S; j++) {
            const float2 v = row[j];
#pragma unroll
            for (int q = 0; q < SEG; q++) {
                const int m = j - q;
                if (m >= 0 && m <= 2 * S) {
                    acc[q].x = fmaf(gxr.g[m], v.x, acc[q].x);
                    acc[q].y = fmaf(gxr.g[m], v.y, acc[q].y);
                }
            }
        }
        const int r = r0 + rl;
        if (r < RYP) {
#pragma unroll
            for (int q = 0; q < SEG; q++) {
                const int col = seg * SEG + q, x = px - S + col;
                const bool keep = col < RX && x >= 0 && x < a.W;
                Rg[(size_t)r * RXP + col] = keep ? acc[q] : make_float2(0.f, 0.f);
            }
        }
    }
}

// One CTA per (tile, wx, part of the wy range).  Lane = column, warps split
// the rows; taps come from the parameter bank with compile-time indices.
template <int S>
__global__ void __launch_bounds__(ProbeGeom<S>::THREADS) wff_probe_kernel(ProbeArgs a, PTaps<float, S> gyA,
                                                                          PTaps<float, S> gyB, PTaps<float, S> gxf)
{
    using G = ProbeGeom<S>;
    constexpr int P = G::P, RXP = G::RXP, KU = G::KU, RYP = G::RYP;
    extern __shared__ __align__(16) float2 psm[];
    float2 *R = psm;                  // [RYP][RXP]
    float2 *U = R + RYP * RXP;        // [UYP][RXP]
    float2 *eys = U + G::UYP * RXP;   // [RYP] phasors e^{-j wy y} of the R rows
    const int t = blockIdx.x, i = blockIdx.y, part = blockIdx.z, tid = threadIdx.x;
    const int lane = tid & 31, w = tid >> 5, cg = w % G::NCG, rg = w / G::NCG;
    const int col = cg * 32 + lane;
    if (a.seed_dev) a.seed = *a.seed_dev;
    const int2 site = probe_site(a, t);
    if (i == 0 && part == 0 && tid == 0) a.sites[t] = site;
    const int py = site.x, px = site.y;
    const float2 *exi = a.ex + (size_t)i * (a.pitch + 2 * kPhasorPad) + kPhasorPad;
    const float thr = *a.thr, thr2 = thr * thr;

    // ---- R of this (tile, wx) from the row pass (L2-resident)
    {
        const float4 *src = reinterpret_cast<const float4 *>(a.rows + ((size_t)t * gridDim.y + i) * G::R_ELEMS);
        float4 *dst = reinterpret_cast<float4 *>(R);
        for (int e = tid; e < (int)(G::R_ELEMS / 2); e += G::THREADS) dst[e] = src[e];
    }

    float2 cacc[G::CPT];
#pragma unroll
    for (int q = 0; q < G::CPT; q++) cacc[q] = make_float2(0.f, 0.f);
    const size_t eys_stride = (size_t)a.H + 2 * kPhasorPad;
    const int k0 = part * a.nfy / a.nsplit, k1 = (part + 1) * a.nfy / a.nsplit;
    const int u0 = rg * KU;
    for (int k = k0; k < k1; k++) {
        const float2 *eyk = a.ey + (size_t)k * eys_stride + kPhasorPad;
        __syncthreads();  // the previous pass 2 is done with U; R is complete
        for (int e = tid; e < RYP; e += G::THREADS) eys[e] = eyk[min(py - 2 * S + e, a.H - 1 + kPhasorPad)];
        __syncthreads();
        // ---- U rows u0 .. u0+KU-1 of this column: first column filter, threshold
        {
            float2 acc[KU];
#pragma unroll
            for (int q = 0; q < KU; q++) acc[q] = make_float2(0.f, 0.f);
#pragma unroll
            for (int j = 0; j < KU + 2 * S; j++) {
                const float2 r = R[(u0 + j) * RXP + col];
                const float2 p = eys[u0 + j];
                const float dx = r.x * p.x - r.y * p.y, dy = r.x * p.y + r.y * p.x;
#pragma unroll
                for (int q = 0; q < KU; q++) {
                    const int m = j - q;
                    if (m >= 0 && m <= 2 * S) {
                        acc[q].x = fmaf(gyA.g[m], dx, acc[q].x);
                        acc[q].y = fmaf(gyA.g[m], dy, acc[q].y);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < KU; q++) {
                const int Y = py - S + u0 + q;
                const bool keep = Y >= 0 && Y < a.H && acc[q].x * acc[q].x + acc[q].y * acc[q].y >= thr2;
                U[(u0 + q) * RXP + col] = keep ? acc[q] : make_float2(0.f, 0.f);
            }
        }
        __syncthreads();
        // ---- C += e^{+j wy y} (second column filter) on the patch rows
#pragma unroll
        for (int q = 0; q < G::CPT; q++) {
            const int r = rg + q * G::NRG;
            if (r < P) {
                float2 c = make_float2(0.f, 0.f);
#pragma unroll
                for (int m = 0; m <= 2 * S; m++) {
                    const float2 v = U[(r + m) * RXP + col];
                    c.x = fmaf(gyB.g[m], v.x, c.x);
                    c.y = fmaf(gyB.g[m], v.y, c.y);
                }
                const float2 p = eys[r + 2 * S];  // row py + r: e^{-j wy y}, multiply by its conjugate
                cacc[q].x += p.x * c.x + p.y * c.y;
                cacc[q].y += p.x * c.y - p.y * c.x;
            }
        }
    }
    __syncthreads();
    float2 *C = U;  // [P][RXP]
#pragma unroll
    for (int q = 0; q < G::CPT; q++) {
        const int r = rg + q * G::NRG;
        if (r < P) C[r * RXP + col] = cacc[q];
    }
    __syncthreads();
    // ---- final row filter and modulation on the P x P patch
    for (int e = tid; e < P * P; e += G::THREADS) {
        const int cy = e / P, cx = e - cy * P;
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int m = 0; m <= 2 * S; m++) {
            const float2 v = C[cy * RXP + cx + m];
            acc.x = fmaf(gxf.g[m], v.x, acc.x);
            acc.y = fmaf(gxf.g[m], v.y, acc.y);
        }
        const float2 p = exi[px + cx];
        a.partial[((size_t)t * gridDim.y * gridDim.z + i * gridDim.z + part) * P * P + e] =
            make_float2(p.x * acc.x + p.y * acc.y, p.x * acc.y - p.y * acc.x);
    }
}

// One block of 256 threads per tile: sum the partials (fixed order), RMS
// phase residual of cmp against the exact patch where |WFF2| >= 0.1.
__global__ void __launch_bounds__(256) wff_probe_resid_kernel(const float2 *__restrict__ partial,
                                                              const int2 *__restrict__ sites, int nparts, int P,
                                                              int W, int H, const float2 *__restrict__ cmp, float tol,
                                                              float *__restrict__ resid, int *__restrict__ flags,
                                                              int *__restrict__ counts, uint32_t *__restrict__ seed)
{
    __shared__ float2 s_part[256];
    __shared__ float s_se[8];
    __shared__ int s_n[8];
    const int t = blockIdx.x, tid = threadIdx.x, PP = P * P;
    // G threads per patch pixel each sum every G-th part (ascending), then
    // the G sums are added in order g = 0 .. G-1: a fixed summation order
    const int G = 256 / PP, e = tid % PP, g = tid / PP;
    float2 v = make_float2(0.f, 0.f);
    if (g < G) {
#pragma unroll 4
        for (int i = g; i < nparts; i += G) {
            const float2 q = partial[((size_t)t * nparts + i) * PP + e];
            v.x += q.x;
            v.y += q.y;
        }
    }
    s_part[tid] = v;
    __syncthreads();
    float se = 0.f;
    int cnt = 0;
    if (tid < PP) {
        float2 sum = s_part[tid];
        for (int k = 1; k < G; k++) {
            sum.x += s_part[k * PP + tid].x;
            sum.y += s_part[k * PP + tid].y;
        }
        const int2 st = sites[t];
        const int y = st.x + tid / P, x = st.y + tid % P;
        if (y < H && x < W && sum.x * sum.x + sum.y * sum.y >= 0.01f) {
            const float2 c = cmp[(size_t)y * W + x];
            const float d = atan2f(c.y * sum.x - c.x * sum.y, c.x * sum.x + c.y * sum.y);
            se = d * d;
            cnt = 1;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        se += __shfl_down_sync(0xffffffffu, se, o);
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    if ((tid & 31) == 0) {
        s_se[tid >> 5] = se;
        s_n[tid >> 5] = cnt;
    }
    __syncthreads();
    if (tid == 0) {
        float sse = 0.f;
        int n = 0;
        for (int k = 0; k < 8; k++) {
            sse += s_se[k];
            n += s_n[k];
        }
        const float r = n ? sqrtf(sse / (float)n) : 0.f;
        resid[t] = r;
        flags[t] = r > tol ? 1 : 0;
        atomicAdd(&counts[0], 1);
        if (r > tol) atomicAdd(&counts[1], 1);
        // the sweep kernels of this frame have read the seed: advance it for the next frame
        if (t == 0 && seed) atomicAdd(seed, 1u);
    }
}

template <int S> static PTaps<float, S> probe_taps(const double *g, int strue, double mul)
{
    PTaps<float, S> t;
    for (int m = 0; m <= 2 * S; m++) {
        const int k = m - S;
        t.g[m] = (k >= -strue && k <= strue) ? (float)(g[k + strue] * mul) : 0.f;
    }
    return t;
}

static int sm_count() { return device_sm_count(); }

template <int S> static int launch_probe_sweep(WffPlan &Pl, ProbeArgs a, cudaStream_t s)
{
    using G = ProbeGeom<S>;
    GLSU_TRY(raise_smem_limit((const void *)wff_probe_kernel<S>, (int)G::SMEM));
    GLSU_TRY(raise_smem_limit((const void *)wff_probe_rows_kernel<S>, (int)G::RSMEM));
    const int ntiles = a.ntx * a.nty;
    // split the wy range (at most 4 parts) so that the last wave of CTAs is well filled
    const int per_sm = (int)((228 * 1024) / (G::SMEM + 1024));
    const int slots = sm_count() * (per_sm > 0 ? per_sm : 1);
    double best = 1e30;
    for (int ns = 1; ns <= 4 && ns <= Pl.nfy; ns++) {
        const long long ctas = (long long)ntiles * Pl.nfx * ns;
        const double cost = (double)((ctas + slots - 1) / slots) * (1.0 / ns + 0.02);
        if (cost < best - 1e-9) {
            best = cost;
            a.nsplit = ns;
        }
    }
    wff_probe_rows_kernel<S><<<dim3(ntiles, Pl.nfx, (G::RYP + G::CR - 1) / G::CR), G::RTHREADS, G::RSMEM, s>>>(
        a, probe_taps<S>(Pl.gx, Pl.sx, 1.0));
    wff_probe_kernel<S><<<dim3(ntiles, Pl.nfx, a.nsplit), G::THREADS, G::SMEM, s>>>(
        a, probe_taps<S>(Pl.gy, Pl.sy, Pl.inv_norm), probe_taps<S>(Pl.gy, Pl.sy, 1.0),
        probe_taps<S>(Pl.gx, Pl.sx, Pl.scale * Pl.inv_norm));
    GLSU_CUDA_TRY(cudaGetLastError());
    Pl.probe_parts = Pl.nfx * a.nsplit;
    Pl.probe_P = G::P;
    Pl.probe_ntiles = ntiles;
    return GLSU_OK;
}

int WffPlan::enqueue_probe_sweep(cudaStream_t s, const void *d_f, int tile, int P, uint32_t seed, const ProbeOut &o)
{
    if (prec != GLSU_F32) return fail(GLSU_ERR_UNSUPPORTED, "the WFF2 probe runs in FP32");
    const int S = std::max(sxi, syi);
    if (S > 45) return fail(GLSU_ERR_UNSUPPORTED, "the WFF2 probe supports window half-sizes up to 45");
    if (P != probe_patch_for_half(S)) return fail(GLSU_ERR_INVALID, "probe patch size does not match the window");
    if (tile < P) return fail(GLSU_ERR_INVALID, "probe patch larger than the tile");
    GLSU_TRY(ensure_threshold(s, d_f));
    ProbeArgs a;
    a.f = (const float2 *)d_f;
    a.ex = (const float2 *)d_ex;
    a.ey = (const float2 *)d_ey;
    a.thr = (const float *)d_thr;
    a.W = W;
    a.H = H;
    a.pitch = pitch;
    a.nfx = nfx;
    a.nfy = nfy;
    a.P = P;
    a.tile = tile;
    a.ntx = (W + tile - 1) / tile;
    a.nty = (H + tile - 1) / tile;
    a.nsplit = 1;
    a.seed = seed;
    a.partial = o.partial;
    a.sites = o.sites;
    a.rows = o.rows;
    a.seed_dev = o.seed;
    if (!o.rows || !o.partial || !o.sites) return fail(GLSU_ERR_INVALID, "probe buffers not allocated");
    switch (S) {
    case 12: return launch_probe_sweep<12>(*this, a, s);
    case 20: return launch_probe_sweep<20>(*this, a, s);
    case 30: return launch_probe_sweep<30>(*this, a, s);
    default: return launch_probe_sweep<45>(*this, a, s);
    }
}

int WffPlan::enqueue_probe_resid(cudaStream_t s, const void *d_cmp, double tol, const ProbeOut &o)
{
    if (probe_parts <= 0) return fail(GLSU_ERR_INVALID, "probe residual without a probe sweep");
    wff_probe_resid_kernel<<<probe_ntiles, 256, 0, s>>>(o.partial, o.sites, probe_parts, probe_P, W, H,
                                                       (const float2 *)d_cmp, (float)tol, o.resid, o.flags, o.counts,
                                                       o.seed);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

int WffPlan::enqueue_probe(cudaStream_t s, const void *d_f, const void *d_cmp, int tile, int P, uint32_t seed,
                           double tol, const ProbeOut &o)
{
    GLSU_TRY(enqueue_probe_sweep(s, d_f, tile, P, seed, o));
    return enqueue_probe_resid(s, d_cmp, tol, o);
}

}  // namespace glsu
