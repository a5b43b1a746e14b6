// wff_colfft.cuh -- WFF2 column sweep with register/shared-memory FFTs (FP32).
//
// Same mathematics as wff_cols_kernel, evaluated in the frequency domain of
// each column.  For one x-frequency plane R_i and one column, with
// h_k(m) = gy(m) e^{j wy_k m} (m in [-s, s]) the truncated, modulated
// window and L >= H + 2s (so the circular convolutions below are the
// linear, zero-boundary ones of the reference):
//     S    = FFT(R)
//     U_k  = IFFT(S . H_k)                   (|U_k| / (L N) is |sf|)
//     T_k  = U_k . [ |U_k| >= L N thr ],  rows >= H set to 0
//     Ch  += FFT(T_k) . H_k                  (sum over wy_k in the spectrum)
//     C    = IFFT(Ch) / (L^2 N)              (the C_i plane of the direct kernel)
// H_k = FFT(h_k) is tabulated exactly (host, FP64), so the window is the
// reference CPU path's truncated one.  Each inverse transform is computed
// as conj(FFT(conj(x))), so one forward transform body serves all
// 2 nfy + 2 transforms of a column.
//
// Layout.  A column is owned by T threads (half a warp to four warps); each
// holds Q = L / T elements in registers in the cyclic order x[t + T m], which
// is both the input order of the first radix pass and the output order of
// the last one (Stockham autosort with butterflies j = t + T q), so the
// window products, the threshold and the spectrum accumulator work in
// registers.  Between passes the data go through a per-column exchange
// buffer in shared memory whose rows are padded so that the 64-bit stores
// and loads of every half-warp fall on distinct banks.  All index
// arithmetic is compile-time (one kernel per transform length); the
// columns of a CTA are independent and synchronise only within a column
// (__syncwarp, or a named barrier when a column spans several warps).
#pragma once

#include <algorithm>

#include "glsu_internal.cuh"

namespace glsu {
namespace colfft {

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }  // a * (-i)

// forward DFTs of 2, 3, 4, 5 and 8 points in registers (exponent -2 pi i / R)
__device__ __forceinline__ void dft2(float2 *v)
{
    const float2 a = v[0], b = v[1];
    v[0] = make_float2(a.x + b.x, a.y + b.y);
    v[1] = make_float2(a.x - b.x, a.y - b.y);
}

__device__ __forceinline__ void dft4(float2 *v)
{
    const float2 a0 = make_float2(v[0].x + v[2].x, v[0].y + v[2].y);
    const float2 a1 = make_float2(v[0].x - v[2].x, v[0].y - v[2].y);
    const float2 a2 = make_float2(v[1].x + v[3].x, v[1].y + v[3].y);
    const float2 a3 = mul_mi(make_float2(v[1].x - v[3].x, v[1].y - v[3].y));
    v[0] = make_float2(a0.x + a2.x, a0.y + a2.y);
    v[2] = make_float2(a0.x - a2.x, a0.y - a2.y);
    v[1] = make_float2(a1.x + a3.x, a1.y + a3.y);
    v[3] = make_float2(a1.x - a3.x, a1.y - a3.y);
}

__device__ __forceinline__ void dft8(float2 *v)
{
    // X[2q] = DFT4(v_r + v_{r+4}), X[2q+1] = DFT4((v_r - v_{r+4}) w8^r), w8 = e^{-i pi/4}
    const float h = 0.70710678118654752f;
    float2 b[4], c[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        b[r] = make_float2(v[r].x + v[r + 4].x, v[r].y + v[r + 4].y);
        c[r] = make_float2(v[r].x - v[r + 4].x, v[r].y - v[r + 4].y);
    }
    c[1] = make_float2(h * (c[1].x + c[1].y), h * (c[1].y - c[1].x));
    c[2] = mul_mi(c[2]);
    c[3] = make_float2(h * (c[3].y - c[3].x), -h * (c[3].x + c[3].y));
    dft4(b);
    dft4(c);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        v[2 * q] = b[q];
        v[2 * q + 1] = c[q];
    }
}

__device__ __forceinline__ void dft3(float2 *v)
{
    const float s3 = 0.86602540378443865f;  // sin(2 pi / 3)
    const float2 t1 = make_float2(v[1].x + v[2].x, v[1].y + v[2].y);
    const float2 t2 = make_float2(v[1].x - v[2].x, v[1].y - v[2].y);
    const float2 m = make_float2(v[0].x - 0.5f * t1.x, v[0].y - 0.5f * t1.y);
    const float2 j = make_float2(s3 * t2.y, -s3 * t2.x);  // -i s3 t2
    v[0] = make_float2(v[0].x + t1.x, v[0].y + t1.y);
    v[1] = make_float2(m.x + j.x, m.y + j.y);
    v[2] = make_float2(m.x - j.x, m.y - j.y);
}

__device__ __forceinline__ void dft5(float2 *v)
{
    const float c1 = 0.30901699437494742f, c2 = -0.80901699437494742f;  // cos(2pi/5), cos(4pi/5)
    const float s1 = 0.95105651629515357f, s2 = 0.58778525229247313f;   // sin(2pi/5), sin(4pi/5)
    const float2 a1 = make_float2(v[1].x + v[4].x, v[1].y + v[4].y);
    const float2 b1 = make_float2(v[1].x - v[4].x, v[1].y - v[4].y);
    const float2 a2 = make_float2(v[2].x + v[3].x, v[2].y + v[3].y);
    const float2 b2 = make_float2(v[2].x - v[3].x, v[2].y - v[3].y);
    const float2 m1 = make_float2(v[0].x + c1 * a1.x + c2 * a2.x, v[0].y + c1 * a1.y + c2 * a2.y);
    const float2 m2 = make_float2(v[0].x + c2 * a1.x + c1 * a2.x, v[0].y + c2 * a1.y + c1 * a2.y);
    const float2 n1 = make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y);
    const float2 n2 = make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y);
    const float2 j1 = make_float2(n1.y, -n1.x);  // -i n1
    const float2 j2 = make_float2(n2.y, -n2.x);
    v[0] = make_float2(v[0].x + a1.x + a2.x, v[0].y + a1.y + a2.y);
    v[1] = make_float2(m1.x + j1.x, m1.y + j1.y);
    v[4] = make_float2(m1.x - j1.x, m1.y - j1.y);
    v[2] = make_float2(m2.x + j2.x, m2.y + j2.y);
    v[3] = make_float2(m2.x - j2.x, m2.y - j2.y);
}

template <int R> __device__ __forceinline__ void dft(float2 *v)
{
    if constexpr (R == 2) dft2(v);
    else if constexpr (R == 4) dft4(v);
    else if constexpr (R == 8) dft8(v);
    else if constexpr (R == 3) dft3(v);
    else dft5(v);
}

// ---------------------------------------------------------------------------
// Compile-time plan of one transform length: L = R0 R1 ... (radix 8 first,
// the one radix 3 or 5 last), T threads per column, Q = L / T elements per
// thread; every radix divides Q.
// ---------------------------------------------------------------------------
template <int L_, int T_, int R0, int R1, int R2, int R3 = 1, int R4 = 1> struct Plan {
    static constexpr int L = L_, T = T_, Q = L_ / T_;
    static constexpr int NP = R4 > 1 ? 5 : (R3 > 1 ? 4 : 3);
    __host__ __device__ static constexpr int radix(int p)
    {
        return p == 0 ? R0 : p == 1 ? R1 : p == 2 ? R2 : p == 3 ? R3 : R4;
    }
    __host__ __device__ static constexpr int ns(int p) { return p == 0 ? 1 : ns(p - 1) * radix(p - 1); }
    // Row length of pass p's exchange buffer (R rows of L/R outputs).  A
    // half-warp's 64-bit accesses use 16 float2 banks; the next pass reads
    // 16 consecutive natural indices, which fall in rows r spaced by this
    // length, so it is padded to 16/R (mod 16) when Ns R < 16 and to Ns
    // (mod 16) when Ns < 16 <= Ns R; with Ns >= 16 a half-warp reads one row.
    __host__ __device__ static constexpr int xrow(int p)
    {
        return (ns(p) >= 16) ? L / radix(p)
                             : L / radix(p) + ((((ns(p) * radix(p) >= 16) ? ns(p) : 16 / radix(p)) -
                                               (L / radix(p)) % 16 + 16) % 16);
    }
    __host__ __device__ static constexpr int xsize(int p) { return radix(p) * xrow(p); }
    __host__ __device__ static constexpr int xbuf_p(int p) { return p >= NP - 1 ? 0 : (xsize(p) > xbuf_p(p + 1) ? xsize(p) : xbuf_p(p + 1)); }
    static constexpr int XBUF = xbuf_p(0);  // float2 of one column's exchange buffer
    static_assert(L_ % T_ == 0 && T_ % 16 == 0, "plan");
    static_assert(Q % R0 == 0 && Q % R1 == 0 && Q % R2 == 0 && Q % R3 == 0 && Q % R4 == 0, "radix must divide Q");
    static_assert(R0 * R1 * R2 * R3 * R4 == L_, "radices must multiply to L");
};

// Synchronise the T threads of one column (column slot col of the CTA).
template <int T> __device__ __forceinline__ void col_sync(int col)
{
    if constexpr (T <= 32) {
        __syncwarp();
    } else {
        asm volatile("bar.sync %0, %1;" ::"r"(1 + col), "n"(T) : "memory");
    }
}

// Radix pass p of the forward transform of one column.  Input: for p = 0
// the registers in cyclic order (v[m] = x[t + T m]); else pass p-1's
// exchange buffer.  Output: pass p's exchange buffer, or for the last pass
// the registers in cyclic order.  tw[e] = e^{-2 pi i e / L}.
template <class P, int p>
__device__ __forceinline__ void pass(float2 (&v)[P::Q], float2 *__restrict__ xb, const float2 *__restrict__ tw, int t,
                                     int col)
{
    constexpr int L = P::L, T = P::T, Q = P::Q, R = P::radix(p), NB = Q / R, Ns = P::ns(p);
    constexpr bool first = p == 0, last = p == P::NP - 1;
    if constexpr (!first) {
        constexpr int Rp = P::radix(p - 1), Nsp = P::ns(p - 1), Xp = P::xrow(p - 1);
#pragma unroll
        for (int q = 0; q < NB; q++)
#pragma unroll
            for (int r = 0; r < R; r++) {
                // natural index n = j + r L/R of input r of butterfly j = t + T q;
                // pass p-1 wrote it as output rp of its butterfly b Nsp + k
                const int n = t + T * q + r * (L / R);
                const int b = n / (Nsp * Rp), rem = n % (Nsp * Rp);
                v[q * R + r] = xb[(rem / Nsp) * Xp + b * Nsp + rem % Nsp];
            }
        col_sync<T>(col);  // every read of the buffer done before this pass writes it
    }
    float2 o[last ? Q : 1];
#pragma unroll
    for (int q = 0; q < NB; q++) {
        float2 a[R];
#pragma unroll
        for (int r = 0; r < R; r++) a[r] = first ? v[q + r * NB] : v[q * R + r];
        if constexpr (Ns > 1) {
            // twiddles w_{Ns R}^{r k}, k = j mod Ns (Ns a power of two)
            const int k = (Ns <= T) ? (t & (Ns - 1)) : (t + T * (q % (Ns > T ? Ns / T : 1)));
#pragma unroll
            for (int r = 1; r < R; r++) a[r] = cmul(a[r], __ldg(tw + r * k * (L / (Ns * R))));
        }
        dft<R>(a);
        if constexpr (last) {
#pragma unroll
            for (int r = 0; r < R; r++) o[q + r * NB] = a[r];  // n = t + T (q + r NB)
        } else {
            const int j = t + T * q;
#pragma unroll
            for (int r = 0; r < R; r++) xb[r * P::xrow(p) + j] = a[r];
        }
    }
    if constexpr (last) {
#pragma unroll
        for (int m = 0; m < Q; m++) v[m] = o[m];
    } else {
        col_sync<T>(col);  // this pass's outputs visible to the column
    }
}

template <class P>
__device__ __forceinline__ void fft(float2 (&v)[P::Q], float2 *__restrict__ xb, const float2 *__restrict__ tw, int t,
                                    int col)
{
    pass<P, 0>(v, xb, tw, t, col);
    pass<P, 1>(v, xb, tw, t, col);
    pass<P, 2>(v, xb, tw, t, col);
    if constexpr (P::NP > 3) pass<P, 3>(v, xb, tw, t, col);
    if constexpr (P::NP > 4) pass<P, 4>(v, xb, tw, t, col);
}

// Shared memory of a CTA of NCOL columns: per column the exchange buffer
// and the spectrum S of the column.
template <class P> constexpr size_t smem_per_column() { return sizeof(float2) * (size_t)(P::XBUF + P::L); }

// ---------------------------------------------------------------------------
// The column sweep.  CTA (g, i): columns g NCOL .. g NCOL + NCOL - 1 of plane
// i (or, in a tile-masked run, column groups list[item] for item = g,
// g + gridDim.x, ...).  One loop runs the 2 nfy + 2 transforms of a column
// through a single transform body.
// ---------------------------------------------------------------------------
// Resident warps per SM the register budget aims at (the spectrum
// accumulator and the working transform take 4 Q floats a thread).
template <class P> constexpr int target_warps() { return P::Q <= 16 ? 16 : P::Q <= 24 ? 12 : P::Q <= 32 ? 10 : 8; }
template <class P, int NCOL> constexpr int min_ctas()
{
    return target_warps<P>() / (P::T * NCOL / 32) > 1 ? target_warps<P>() / (P::T * NCOL / 32) : 1;
}

// Geometry of the columns a CTA sweeps: one plane's input and output, the
// window spectra, threshold and scale, and the CTA's first column.  It sits
// in shared memory and is re-read where used, so that none of it occupies
// registers across the transforms (the batched kernel below takes it from a
// table with a run-time index; kept in registers it would spill).
struct SweepGeom {
    const float2 *R;
    float2 *C;
    const float2 *khat;
    float thr2, out_scale;
    int H, pitch, nfy, x0;
};
template <typename T> __device__ __forceinline__ T vld(const T &r) { return *(const volatile T *)&r; }

// The 2 nfy + 2 transforms of column x0 + col of one plane, run by the T
// threads (t) of column slot col through a single transform body.  Both
// kernels below run every column through this function, so a column's
// outputs are the same bits whichever kernel ran it.
template <class P>
__device__ __forceinline__ void sweep_column(const SweepGeom &g, const float2 *__restrict__ tw,
                                             float2 *__restrict__ xb, float2 *__restrict__ S, int t, int col)
{
    constexpr int L = P::L, T = P::T, Q = P::Q;
    const int nit = 2 * vld(g.nfy) + 2;
    float2 v[Q], ch[Q];
#pragma unroll 1
    for (int it = 0; it < nit; it++) {
        const int k = (it - 1) >> 1;  // wy index of the inverse (odd it) / forward (even it >= 2) pair
        if (it == 0) {
            const float2 *Ri = vld(g.R);
            const int H = vld(g.H), pitch = vld(g.pitch), x = vld(g.x0) + col;
#pragma unroll
            for (int m = 0; m < Q; m++) {
                const int row = t + T * m;
                v[m] = row < H ? Ri[(size_t)row * pitch + x] : make_float2(0.f, 0.f);
            }
        } else if (it == nit - 1) {
#pragma unroll
            for (int m = 0; m < Q; m++) v[m] = conjf2(ch[m]);
        } else if (it & 1) {
            const float2 *hk = vld(g.khat) + (size_t)k * L;
#pragma unroll
            for (int m = 0; m < Q; m++) v[m] = conjf2(cmul(S[t + T * m], __ldg(hk + t + T * m)));
        }
        fft<P>(v, xb, tw, t, col);
        if (it == 0) {
#pragma unroll
            for (int m = 0; m < Q; m++) {
                S[t + T * m] = v[m];  // read back only by this thread
                ch[m] = make_float2(0.f, 0.f);
            }
        } else if (it == nit - 1) {
            float2 *Ci = vld(g.C);
            const int H = vld(g.H), pitch = vld(g.pitch), x = vld(g.x0) + col;
            const float out_scale = vld(g.out_scale);
#pragma unroll
            for (int m = 0; m < Q; m++) {
                const int row = t + T * m;
                if (row < H) Ci[(size_t)row * pitch + x] = make_float2(v[m].x * out_scale, -v[m].y * out_scale);
            }
        } else if (it & 1) {
            // u = conj(v): hard threshold in the spatial domain, rows >= H dropped
            const int H = vld(g.H);
            const float thr2 = vld(g.thr2);
#pragma unroll
            for (int m = 0; m < Q; m++) {
                const int row = t + T * m;
                const float2 u = conjf2(v[m]);
                const bool keep = row < H && (u.x * u.x + u.y * u.y >= thr2);
                v[m] = keep ? u : make_float2(0.f, 0.f);
            }
        } else {
            const float2 *hk = vld(g.khat) + (size_t)k * L;
#pragma unroll
            for (int m = 0; m < Q; m++) {
                const float2 a = v[m], h = __ldg(hk + t + T * m);
                ch[m].x += a.x * h.x - a.y * h.y;
                ch[m].y += a.x * h.y + a.y * h.x;
            }
        }
    }
}

template <class P, int NCOL>
__global__ void __launch_bounds__(P::T *NCOL, (min_ctas<P, NCOL>())) wff_colfft_kernel(const float2 *__restrict__ R, float2 *__restrict__ Cout,
                                                               int H, int pitch, int nfy,
                                                               const float2 *__restrict__ khat,
                                                               const float2 *__restrict__ tw,
                                                               const float *__restrict__ thr_ptr, float LN,
                                                               float out_scale, const int2 *__restrict__ list,
                                                               const int *__restrict__ list_count)
{
    constexpr int L = P::L, T = P::T;
    extern __shared__ __align__(16) float2 cf_smem[];
    __shared__ SweepGeom geom;
    const int col = threadIdx.x / T, t = threadIdx.x % T;
    float2 *xb = cf_smem + (size_t)col * (P::XBUF + L);
    float2 *S = xb + P::XBUF;
    const int nitems = list ? *list_count : (int)gridDim.x;
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        __syncthreads();  // every column is done with the previous item's geometry
        if (threadIdx.x == 0) {
            const size_t plane = (size_t)H * pitch;
            const float thr = LN * (*thr_ptr);
            geom = SweepGeom{R + blockIdx.y * plane, Cout + blockIdx.y * plane, khat, thr * thr, out_scale,
                             H, pitch, nfy, (list ? list[item].x : item) * NCOL};
        }
        __syncthreads();
        sweep_column<P>(geom, tw, xb, S, t, col);
    }
}

// One sequence of a batched column sweep (glsu_dpra_batch): its planes, its
// window spectra and threshold, and where its items start in the batch's
// work list.  Sequence s owns items item0[s] .. item0[s+1] - 1, item
// (plane i, column group g) = item0 + i * ngroups + g.  The table travels
// as a kernel parameter (constant bank).
constexpr int kMaxBatchSeqs = 128;
struct BatchSeq {
    const float2 *R;
    float2 *C;
    const float2 *khat;
    const float *thr;
    int H, pitch, nfy, ngroups;
    float LN, out_scale;
    int item0;
    int pad_;
};
struct BatchTable {
    BatchSeq seq[kMaxBatchSeqs];
};

// The column sweep of many sequences of one transform length in one
// persistent launch: each CTA walks the batch's work list of (sequence,
// plane, column group) items with stride gridDim.x.
template <class P, int NCOL>
__global__ void __launch_bounds__(P::T *NCOL, (min_ctas<P, NCOL>()))
    wff_colfft_batch_kernel(const __grid_constant__ BatchTable tab, int nseq, int nitems,
                            const float2 *__restrict__ tw)
{
    constexpr int L = P::L, T = P::T;
    extern __shared__ __align__(16) float2 cf_smem[];
    __shared__ SweepGeom geom;
    const int col = threadIdx.x / T, t = threadIdx.x % T;
    float2 *xb = cf_smem + (size_t)col * (P::XBUF + L);
    float2 *S = xb + P::XBUF;
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        __syncthreads();  // every column is done with the previous item's geometry
        if (threadIdx.x == 0) {
            int lo = 0, hi = nseq - 1;  // the last sequence with item0 <= item
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (tab.seq[mid].item0 <= item) lo = mid;
                else hi = mid - 1;
            }
            const BatchSeq &q = tab.seq[lo];
            const int local = item - q.item0;
            const int i = local / q.ngroups, g = local - i * q.ngroups;
            const size_t plane = (size_t)q.H * q.pitch;
            const float thr = q.LN * (*q.thr);
            geom = SweepGeom{q.R + i * plane, q.C + i * plane, q.khat, thr * thr, q.out_scale, q.H, q.pitch, q.nfy,
                             g * NCOL};
        }
        __syncthreads();
        sweep_column<P>(geom, tw, xb, S, t, col);
    }
}

// Transform lengths with a compiled plan, ascending.
constexpr int kLengths[] = {256, 384, 512, 640, 768, 1024, 1280, 1536, 2048, 2560, 3072, 4096};
constexpr int kNumLengths = sizeof(kLengths) / sizeof(kLengths[0]);

}  // namespace colfft
}  // namespace glsu

namespace glsu {
namespace colfft {

// Launch the sweep of plan P with NCOL columns per CTA; list/count: the
// device list of column groups of a tile-masked run (null: all groups).
template <class P, int NCOL>
int launch(const WffPlan &Pl, cudaStream_t s, const int2 *list, const int *count, int grid_x)
{
    const size_t smem = NCOL * smem_per_column<P>();
    GLSU_TRY(raise_smem_limit((const void *)wff_colfft_kernel<P, NCOL>, (int)smem));
    const double N = 1.0 / Pl.inv_norm;
    dim3 grid(grid_x, Pl.nfx);
    wff_colfft_kernel<P, NCOL><<<grid, P::T * NCOL, smem, s>>>(
        (const float2 *)Pl.d_R, (float2 *)Pl.d_C, Pl.H, Pl.pitch, Pl.nfy, (const float2 *)Pl.d_khat,
        (const float2 *)Pl.d_tw, (const float *)Pl.d_thr, (float)(P::L * N),
        (float)(1.0 / ((double)P::L * P::L * N)), list, count);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

// Launch the batched sweep of plan P (default CTA width NCOL) over nitems
// items of nseq sequences (device array seqs), grid_x persistent CTAs.
template <class P, int NCOL>
int launch_batch(const BatchTable &tab, int nseq, int nitems, const float2 *tw, int grid_x, cudaStream_t s)
{
    const size_t smem = NCOL * smem_per_column<P>();
    GLSU_TRY(raise_smem_limit((const void *)wff_colfft_batch_kernel<P, NCOL>, (int)smem));
    if (grid_x <= 0) {  // persistent: as many CTAs as are resident at once
        int per_sm = 0;
        GLSU_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wff_colfft_batch_kernel<P, NCOL>,
                                                                    P::T * NCOL, smem));
        grid_x = std::max(1, per_sm) * device_sm_count();
    }
    grid_x = std::max(1, std::min(grid_x, nitems));
    wff_colfft_batch_kernel<P, NCOL><<<grid_x, P::T * NCOL, smem, s>>>(tab, nseq, nitems, tw);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

// Per transform length: its plan, and the two CTA widths compiled for it
// (the default first).  Each length group lives in its own translation unit
// so that they compile in parallel; each returns GLSU_ERR_UNSUPPORTED for
// lengths it does not hold.
int launch_len_small(int L, int ncol, const WffPlan &Pl, cudaStream_t s, const int2 *list, const int *count,
                     int grid_x);
int launch_len_mid(int L, int ncol, const WffPlan &Pl, cudaStream_t s, const int2 *list, const int *count,
                   int grid_x);
int launch_len_large(int L, int ncol, const WffPlan &Pl, cudaStream_t s, const int2 *list, const int *count,
                     int grid_x);
// The batched sweep at the length's default CTA width (same grouping).
int launch_batch_small(int L, const BatchTable &tab, int nseq, int nitems, const float2 *tw, int grid_x,
                       cudaStream_t s);
int launch_batch_mid(int L, const BatchTable &tab, int nseq, int nitems, const float2 *tw, int grid_x,
                     cudaStream_t s);
int launch_batch_large(int L, const BatchTable &tab, int nseq, int nitems, const float2 *tw, int grid_x,
                       cudaStream_t s);

// Threads per column, passes and shared memory per column of each length
// (host-side mirror of the plans).
struct LenInfo {
    int L, T, passes, ncol_default;
    size_t smem_col;
};
bool len_info(int L, LenInfo *out);

}  // namespace colfft
}  // namespace glsu

#define GLSU_COLFFT_BATCH_CASE(LEN, PLAN, NC0) \
    case LEN:                                   \
        return launch_batch<PLAN, NC0>(tab, nseq, nitems, tw, grid_x, s);

#define GLSU_COLFFT_CASE(LEN, PLAN, NC0)                                                            \
    case LEN: {                                                                                     \
        using P_ = PLAN;                                                                            \
        if (ncol == NC0) return launch<P_, NC0>(Pl, s, list, count, grid_x);                        \
        if (ncol == 2 * NC0 && 2 * NC0 * P_::T <= 512 && 2 * NC0 * smem_per_column<P_>() <= 227 * 1024) \
            return launch<P_, (2 * NC0 * P_::T <= 512 ? 2 * NC0 : NC0)>(Pl, s, list, count, grid_x); \
        return fail(GLSU_ERR_UNSUPPORTED, "column FFT: CTA width not compiled for this length");   \
    }
