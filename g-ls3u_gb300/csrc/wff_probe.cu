// wff_probe.cu -- exact WFF2 on sparse patches: the judge of the surrogate.
//
// For each tile of the frame, one P x P patch (position hashed from a seed
// and the tile index) gets the exact FP32 WFF2 output, computed by the same
// separable, demodulated formulation as the full-frame kernels (rows demod,
// column sweep with threshold, final rows; WFT/WFT2_CPU.cpp:190-390):
// one CTA per (tile, wx), holding in shared memory
//   R  the row-filtered, demodulated input over rows py-2sy .. py+P+2sy-1
//      and columns px-sx .. px+P+sx-1 (zero outside the image, the crop),
//   U  the thresholded first column filter over rows py-sy .. py+P+sy-1,
//   C  the second column filter summed over wy on rows py .. py+P-1,
// then the final row filter on the P x P patch.  The per-wx partials are
// summed in a fixed order by the residual kernel, which compares the patch
// with the surrogate's output and flags the tile.
#include <cmath>

#include "glsu_internal.cuh"

namespace glsu {

constexpr int kProbeTapC = kMaxHalf;  // taps are stored centred at index 60
constexpr int kProbeFR = 8;           // input rows staged per pass of the row filter

struct ProbeTaps {
    float gxr[2 * kMaxHalf + 1];  // row filter of the input (x1)
    float gyA[2 * kMaxHalf + 1];  // first column filter (x 1/norm)
    float gyB[2 * kMaxHalf + 1];  // second column filter (x1)
    float gxf[2 * kMaxHalf + 1];  // final row filter (x scale/norm)
};

struct ProbeArgs {
    const float2 *f, *ex, *ey;
    const float *thr;
    int W, H, pitch, nfx, nfy, sx, sy, P;
    int tile, ntx, nty;
    uint32_t seed;
    float2 *partial;
    int2 *sites;
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

static int probe_smem_floats2(int P, int sx, int sy)
{
    const int RX = P + 2 * sx, RY = P + 4 * sy, UY = P + 2 * sy, FX = P + 4 * sx;
    const int ureg = UY * RX > kProbeFR * FX + FX ? UY * RX : kProbeFR * FX + FX;
    return RY * RX + ureg + P * RX;
}

__global__ void __launch_bounds__(256) wff_probe_kernel(ProbeArgs a, ProbeTaps tp)
{
    extern __shared__ __align__(16) float2 psm[];
    const int t = blockIdx.x, i = blockIdx.y, tid = threadIdx.x;
    const int P = a.P, sx = a.sx, sy = a.sy;
    const int RX = P + 2 * sx, RY = P + 4 * sy, UY = P + 2 * sy, FX = P + 4 * sx;
    float2 *R = psm;
    float2 *U = R + RY * RX;
    float2 *C = U + (UY * RX > kProbeFR * FX + FX ? UY * RX : kProbeFR * FX + FX);
    const int2 site = probe_site(a, t);
    if (i == 0 && tid == 0) a.sites[t] = site;
    const int py = site.x, px = site.y;
    const float2 *exi = a.ex + (size_t)i * (a.pitch + 2 * kPhasorPad) + kPhasorPad;
    const float thr = *a.thr, thr2 = thr * thr;

    // ---- R: rows py-2sy .., demodulated by e^{-j wx x}, filtered along x
    float2 *fs = U;                   // [kProbeFR][FX] staged, demodulated input
    float2 *es = U + kProbeFR * FX;   // [FX] phasors of the staged columns
    for (int e = tid; e < FX; e += 256) es[e] = exi[px - 2 * sx + e];
    for (int r0 = 0; r0 < RY; r0 += kProbeFR) {
        __syncthreads();
        for (int e = tid; e < kProbeFR * FX; e += 256) {
            const int rr = e / FX, c = e - rr * FX;
            const int y = py - 2 * sy + r0 + rr, x = px - 2 * sx + c;
            float2 v = make_float2(0.f, 0.f);
            if (r0 + rr < RY && y >= 0 && y < a.H && x >= 0 && x < a.W) v = a.f[(size_t)y * a.W + x];
            const float2 p = es[c];
            fs[e] = make_float2(v.x * p.x - v.y * p.y, v.x * p.y + v.y * p.x);
        }
        __syncthreads();
        for (int e = tid; e < kProbeFR * RX; e += 256) {
            const int rr = e / RX, c = e - rr * RX;
            if (r0 + rr >= RY) continue;
            const int x = px - sx + c;
            float2 acc = make_float2(0.f, 0.f);
            if (x >= 0 && x < a.W) {
                const float2 *row = fs + rr * FX + c;
                for (int m = 0; m <= 2 * sx; m++) {
                    const float g = tp.gxr[kProbeTapC - sx + m];
                    acc.x = fmaf(g, row[m].x, acc.x);
                    acc.y = fmaf(g, row[m].y, acc.y);
                }
            }
            R[(r0 + rr) * RX + c] = acc;
        }
    }
    for (int e = tid; e < P * RX; e += 256) C[e] = make_float2(0.f, 0.f);

    const size_t eys = (size_t)a.H + 2 * kPhasorPad;
    const int nub = (UY + 3) / 4;
    for (int k = 0; k < a.nfy; k++) {
        const float2 *eyk = a.ey + (size_t)k * eys + kPhasorPad;
        __syncthreads();
        // ---- U: first column filter (4 rows per thread), threshold
        for (int e = tid; e < nub * RX; e += 256) {
            const int c = e % RX, u0 = (e / RX) * 4;
            float2 acc[4];
#pragma unroll
            for (int q = 0; q < 4; q++) acc[q] = make_float2(0.f, 0.f);
            const int jend = min(u0 + 3 + 2 * sy, RY - 1);
            for (int j = u0; j <= jend; j++) {
                const float2 r = R[j * RX + c];
                const float2 p = eyk[py - 2 * sy + j];
                const float dx = r.x * p.x - r.y * p.y, dy = r.x * p.y + r.y * p.x;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int m = j - u0 - q;
                    if (m >= 0 && m <= 2 * sy) {
                        const float g = tp.gyA[kProbeTapC - sy + m];
                        acc[q].x = fmaf(g, dx, acc[q].x);
                        acc[q].y = fmaf(g, dy, acc[q].y);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int uy = u0 + q;
                if (uy >= UY) break;
                const int Y = py - sy + uy;
                const bool keep = Y >= 0 && Y < a.H && acc[q].x * acc[q].x + acc[q].y * acc[q].y >= thr2;
                U[uy * RX + c] = keep ? acc[q] : make_float2(0.f, 0.f);
            }
        }
        __syncthreads();
        // ---- C += e^{+j wy y} (second column filter)
        for (int e = tid; e < P * RX; e += 256) {
            const int cy = e / RX, c = e - cy * RX;
            float2 acc = make_float2(0.f, 0.f);
            for (int j = 0; j <= 2 * sy; j++) {
                const float g = tp.gyB[kProbeTapC - sy + j];
                const float2 v = U[(cy + j) * RX + c];
                acc.x = fmaf(g, v.x, acc.x);
                acc.y = fmaf(g, v.y, acc.y);
            }
            const int Y = min(py + cy, a.H - 1 + kPhasorPad);
            const float2 p = eyk[Y];  // e^{-j wy y}; multiply by its conjugate
            C[e].x += p.x * acc.x + p.y * acc.y;
            C[e].y += p.x * acc.y - p.y * acc.x;
        }
    }
    __syncthreads();
    // ---- final row filter and modulation on the P x P patch
    for (int e = tid; e < P * P; e += 256) {
        const int cy = e / P, cx = e - cy * P;
        float2 acc = make_float2(0.f, 0.f);
        for (int j = 0; j <= 2 * sx; j++) {
            const float g = tp.gxf[kProbeTapC - sx + j];
            const float2 v = C[cy * RX + cx + j];
            acc.x = fmaf(g, v.x, acc.x);
            acc.y = fmaf(g, v.y, acc.y);
        }
        const float2 p = exi[px + cx];
        a.partial[((size_t)t * a.nfx + i) * P * P + e] =
            make_float2(p.x * acc.x + p.y * acc.y, p.x * acc.y - p.y * acc.x);
    }
}

// One block of 64 threads per tile: sum the per-wx partials (fixed order),
// RMS phase residual of cmp against the exact patch where |WFF2| >= 0.1.
__global__ void __launch_bounds__(64) wff_probe_resid_kernel(const float2 *__restrict__ partial,
                                                             const int2 *__restrict__ sites, int nfx, int P, int W,
                                                             int H, const float2 *__restrict__ cmp, float tol,
                                                             float *__restrict__ resid, int *__restrict__ flags,
                                                             int *__restrict__ counts)
{
    __shared__ float s_se[2];
    __shared__ int s_n[2];
    const int t = blockIdx.x, e = threadIdx.x;
    float se = 0.f;
    int cnt = 0;
    if (e < P * P) {
        float2 v = make_float2(0.f, 0.f);
        for (int i = 0; i < nfx; i++) {
            const float2 q = partial[((size_t)t * nfx + i) * P * P + e];
            v.x += q.x;
            v.y += q.y;
        }
        const int2 s = sites[t];
        const int y = s.x + e / P, x = s.y + e % P;
        if (y < H && x < W && v.x * v.x + v.y * v.y >= 0.01f) {
            const float2 c = cmp[(size_t)y * W + x];
            const float d = atan2f(c.y * v.x - c.x * v.y, c.x * v.x + c.y * v.y);
            se = d * d;
            cnt = 1;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        se += __shfl_down_sync(0xffffffffu, se, o);
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    if ((e & 31) == 0) {
        s_se[e >> 5] = se;
        s_n[e >> 5] = cnt;
    }
    __syncthreads();
    if (e == 0) {
        const int n = s_n[0] + s_n[1];
        const float r = n ? sqrtf((s_se[0] + s_se[1]) / (float)n) : 0.f;
        resid[t] = r;
        flags[t] = r > tol ? 1 : 0;
        atomicAdd(&counts[0], 1);
        if (r > tol) atomicAdd(&counts[1], 1);
    }
}

int WffPlan::enqueue_probe(cudaStream_t s, const void *d_f, const void *d_cmp, int tile, int P, uint32_t seed,
                           double tol, const ProbeOut &o)
{
    if (prec != GLSU_F32) return fail(GLSU_ERR_UNSUPPORTED, "the WFF2 probe runs in FP32");
    if (P < 1 || P > kProbeMaxP || tile < P) return fail(GLSU_ERR_INVALID, "probe patch must be 1..8 and <= tile");
    const int smem = (int)(probe_smem_floats2(P, sx, sy) * sizeof(float2));
    if (smem > 227 * 1024) return fail(GLSU_ERR_UNSUPPORTED, "probe patch too large for this window (use P = 4)");
    GLSU_TRY(ensure_threshold(s, d_f));
    static int attr = 0;
    if (smem > attr) {
        GLSU_CUDA_TRY(cudaFuncSetAttribute(wff_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = smem;
    }
    ProbeTaps tp;
    for (int m = -kMaxHalf; m <= kMaxHalf; m++) {
        const bool inx = m >= -sx && m <= sx, iny = m >= -sy && m <= sy;
        tp.gxr[m + kProbeTapC] = inx ? (float)gx[m + sx] : 0.f;
        tp.gxf[m + kProbeTapC] = inx ? (float)(gx[m + sx] * scale * inv_norm) : 0.f;
        tp.gyA[m + kProbeTapC] = iny ? (float)(gy[m + sy] * inv_norm) : 0.f;
        tp.gyB[m + kProbeTapC] = iny ? (float)gy[m + sy] : 0.f;
    }
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
    a.sx = sx;
    a.sy = sy;
    a.P = P;
    a.tile = tile;
    a.ntx = (W + tile - 1) / tile;
    a.nty = (H + tile - 1) / tile;
    a.seed = seed;
    a.partial = o.partial;
    a.sites = o.sites;
    const int ntiles = a.ntx * a.nty;
    wff_probe_kernel<<<dim3(ntiles, nfx), 256, smem, s>>>(a, tp);
    wff_probe_resid_kernel<<<ntiles, 64, 0, s>>>(o.partial, o.sites, nfx, P, W, H, (const float2 *)d_cmp,
                                                 (float)tol, o.resid, o.flags, o.counts);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

}  // namespace glsu
