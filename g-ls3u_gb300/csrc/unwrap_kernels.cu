// unwrap_kernels.cu -- line-scanning spatial phase unwrapping on sm_103a.
//
// MatLab/fp_unwrapping.m:41-71 (which G-LS3U applies to each frame's phase
// change, MatLab/fp_ls3u.m:104; the C++ reference leaves it out): the seed
// column is unwrapped from the start row, then every row from the start
// column, each step adding round((p[i-1] - p[i]) / 2pi) * 2pi to p[i] using the
// already unwrapped neighbour.  Because the neighbour's correction is a whole
// multiple of 2pi, the unwrapped value is p[i] + 2pi K[i] with K a running sum
// of round((p[i-1] - p[i]) / 2pi) over the wrapped input -- a prefix sum, so
// each line is one CTA: chunked jump counts, a block-wide scan, then writes.
#include <cmath>

#include "glsu_internal.cuh"

namespace glsu {

constexpr int kUnwrapThreads = 256;
constexpr int kUnwrapMaxChunk = 16;  // lines up to 4096 elements

__device__ __forceinline__ int block_exclusive_scan(int v, int *warp_sums, int *total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = lane < kUnwrapThreads / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kUnwrapThreads / 32) warp_sums[lane] = s;  // inclusive warp prefix
        if (lane == kUnwrapThreads / 32 - 1) *total = s;
    }
    __syncthreads();
    const int before = (w > 0 ? warp_sums[w - 1] : 0) + x - v;
    __syncthreads();
    return before;
}

// Lines l = blockIdx.x: elements base + l*line_stride + i*elem_stride,
// i in [0, len); unwrapped outward from index s.  add (optional, same
// layout) is added to every output element.
template <typename T>
__global__ void __launch_bounds__(kUnwrapThreads) unwrap_lines_kernel(T *__restrict__ p, const T *__restrict__ add,
                                                                      int len, size_t line_stride,
                                                                      size_t elem_stride, int s)
{
    __shared__ int warp_sums[kUnwrapThreads / 32];
    __shared__ int tot_r, tot_l;
    const T two_pi = (T)6.283185307179586476925286766559;
    const size_t base = (size_t)blockIdx.x * line_stride;
    const int chunk = (len + kUnwrapThreads - 1) / kUnwrapThreads;
    const int i0 = threadIdx.x * chunk;
    T val[kUnwrapMaxChunk];
    int jr[kUnwrapMaxChunk], jl[kUnwrapMaxChunk];
    int sum_r = 0, sum_l = 0;
#pragma unroll
    for (int c = 0; c < kUnwrapMaxChunk; c++) {
        const int i = i0 + c;
        jr[c] = 0;
        jl[c] = 0;
        val[c] = 0;
        if (c < chunk && i < len) {
            const T v = p[base + (size_t)i * elem_stride];
            val[c] = v;
            if (i > s) jr[c] = (int)round((p[base + (size_t)(i - 1) * elem_stride] - v) / two_pi);
            if (i < s) jl[c] = (int)round((p[base + (size_t)(i + 1) * elem_stride] - v) / two_pi);
            sum_r += jr[c];
            sum_l += jl[c];
        }
    }
    // K[i] (i > s) = sum of jr over (s, i];  K[i] (i < s) = sum of jl over [i, s)
    const int pre_r = block_exclusive_scan(sum_r, warp_sums, &tot_r);
    const int pre_l = block_exclusive_scan(sum_l, warp_sums, &tot_l);
    const int total_l = tot_l;
    int kr = pre_r, kl = pre_l;  // running sums before this thread's chunk
#pragma unroll
    for (int c = 0; c < kUnwrapMaxChunk; c++) {
        const int i = i0 + c;
        if (c < chunk && i < len) {
            kr += jr[c];
            int K = 0;
            if (i > s) K = kr;
            if (i < s) K = total_l - kl;  // sum of jl over [i, s)
            kl += jl[c];
            T out = val[c] + two_pi * (T)K;
            if (add) out += add[base + (size_t)i * elem_stride];
            p[base + (size_t)i * elem_stride] = out;
        }
    }
}

template <typename T>
static int unwrap_t(T *d_p, const T *d_add, int W, int H, int row0, int col0, cudaStream_t s)
{
    // seed column col0, from row0 (in place, nothing added)
    unwrap_lines_kernel<T><<<1, kUnwrapThreads, 0, s>>>(d_p + col0, nullptr, H, 0, (size_t)W, row0);
    // every row from col0
    unwrap_lines_kernel<T><<<H, kUnwrapThreads, 0, s>>>(d_p, d_add, W, (size_t)W, 1, col0);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

int launch_unwrap(int prec, void *d_p, const void *d_add, int W, int H, int row0, int col0, cudaStream_t s)
{
    if (W < 1 || H < 1 || W > kUnwrapThreads * kUnwrapMaxChunk || H > kUnwrapThreads * kUnwrapMaxChunk)
        return fail(GLSU_ERR_INVALID, "unwrap: image sides must be 1..4096");
    if (row0 < 0) row0 = (int)std::floor(H / 2.0 + 0.5) - 1;  // MATLAB round(m/2), 1-based
    if (col0 < 0) col0 = (int)std::floor(W / 2.0 + 0.5) - 1;
    if (row0 < 0) row0 = 0;
    if (col0 < 0) col0 = 0;
    if (row0 >= H || col0 >= W) return fail(GLSU_ERR_INVALID, "unwrap: start point outside the image");
    if (prec == GLSU_F32) return unwrap_t<float>((float *)d_p, (const float *)d_add, W, H, row0, col0, s);
    if (prec == GLSU_F64) return unwrap_t<double>((double *)d_p, (const double *)d_add, W, H, row0, col0, s);
    return fail(GLSU_ERR_INVALID, "precision must be F32 or F64");
}

}  // namespace glsu
