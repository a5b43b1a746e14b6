// aia_kernels.cu -- AIA (advanced iterative algorithm) on sm_103a.
//
// Reference: AIA/aia_cpu.cpp:16-263 (CPU) and AIA/aia_cudaf.cu:308-505 (GPU);
// MATLAB definition MatLab/fp_aia.m:50-121.  Each iteration alternates
//   phi-step: per pixel, A1 x = [sum I, sum I cos d, sum I sin d] with A1 built
//             from the frame shifts d only, phi = atan2(-x3, x2);
//   d-step:   per frame, A2 y = [sum I, sum I cos phi, sum I sin phi] with A2
//             built from cos/sin phi summed over all pixels, d = atan2(-y3, y2).
// One fused pass per iteration does the phi-step and accumulates every sum
// the d-step needs (FP64, per-block partials reduced in a fixed order, so the
// result is deterministic); a one-block kernel solves the 3x3 d-step on the
// device and raises a done flag when max|d - d_old| <= tol or the iteration
// cap is hit.  The host enqueues all iterations without synchronising;
// passes after the done flag return at once.
#include <cmath>

#include "glsu_internal.cuh"

namespace glsu {

constexpr int kAiaMaxM = 32;
constexpr int kAiaThreads = 256;

// state layout (doubles): [0,M) deltas, [M,2M) old deltas, [2M] err, [2M+1] iterations,
// [2M+2] status (0 ok, else GLSU_ERR_NOT_POSDEF)
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <typename IMG, int MM>
__global__ void __launch_bounds__(kAiaThreads)
    aia_pass_kernel(const IMG *__restrict__ f, int M, int N, const double *__restrict__ state,
                    const int *__restrict__ done, double *__restrict__ part, int final_pass, float *__restrict__ phi)
{
    if (!final_pass && *done) return;
    __shared__ float cdl[MM], sdl[MM];
    __shared__ double adj[2][3];  // rows 2 and 3 of adj(A1), signed by det(A1)
    __shared__ double red[kAiaThreads / 32][5 + 3 * MM];
    const int tid = threadIdx.x;
    if (tid == 0) {
        double a3 = 0, a4 = 0, a6 = 0, a7 = 0, a8 = 0;
        for (int i = 0; i < M; i++) {
            double s, c;
            sincos(state[i], &s, &c);
            cdl[i] = (float)c;
            sdl[i] = (float)s;
            a3 += c; a4 += c * c; a6 += s; a7 += c * s; a8 += s * s;
        }
        const double A[3][3] = {{(double)M, a3, a6}, {a3, a4, a7}, {a6, a7, a8}};
        // cofactor rows 2,3 of the inverse: x = adj(A) b / det(A)
        const double c10 = -(A[0][1] * A[2][2] - A[0][2] * A[2][1]);
        const double c11 = (A[0][0] * A[2][2] - A[0][2] * A[2][0]);
        const double c12 = -(A[0][0] * A[2][1] - A[0][1] * A[2][0]);
        const double c20 = (A[0][1] * A[1][2] - A[0][2] * A[1][1]);
        const double c21 = -(A[0][0] * A[1][2] - A[0][2] * A[1][0]);
        const double c22 = (A[0][0] * A[1][1] - A[0][1] * A[1][0]);
        const double det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
                           A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                           A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
        const double sg = det < 0 ? -1.0 : 1.0;
        adj[0][0] = sg * c10; adj[0][1] = sg * c11; adj[0][2] = sg * c12;
        adj[1][0] = sg * c20; adj[1][1] = sg * c21; adj[1][2] = sg * c22;
    }
    __syncthreads();
    double acc[5 + 3 * MM];
#pragma unroll
    for (int v = 0; v < 5 + 3 * MM; v++) acc[v] = 0;
    const double a10 = adj[0][0], a11 = adj[0][1], a12 = adj[0][2];
    const double a20 = adj[1][0], a21 = adj[1][1], a22 = adj[1][2];
    for (int j = blockIdx.x * kAiaThreads + tid; j < N; j += gridDim.x * kAiaThreads) {
        float I[MM];
        float b0 = 0, b1 = 0, b2 = 0;
#pragma unroll
        for (int i = 0; i < MM; i++) {
            I[i] = 0;
            if (i < M) {
                I[i] = (float)f[(size_t)i * N + j];
                b0 += I[i];
                b1 = fmaf(I[i], cdl[i], b1);
                b2 = fmaf(I[i], sdl[i], b2);
            }
        }
        const double X = a10 * b0 + a11 * b1 + a12 * b2;  // ~ x2
        const double Y = a20 * b0 + a21 * b1 + a22 * b2;  // ~ x3
        if (final_pass) {
            double p = atan2(-Y, X) + state[0];
            double s, c;
            sincos(p, &s, &c);
            phi[j] = (float)atan2(s, c);
            continue;
        }
        const double h = hypot(X, Y);
        const double c = h > 0 ? X / h : 1.0, s = h > 0 ? -Y / h : 0.0;
        acc[0] += c; acc[1] += c * c; acc[2] += s; acc[3] += c * s; acc[4] += s * s;
#pragma unroll
        for (int i = 0; i < MM; i++) {
            if (i < M) {
                acc[5 + 3 * i] += I[i];
                acc[6 + 3 * i] += I[i] * c;
                acc[7 + 3 * i] += I[i] * s;
            }
        }
    }
    if (final_pass) return;
    const int lane = tid & 31, wid = tid >> 5;
    const int nv = 5 + 3 * M;
#pragma unroll
    for (int v = 0; v < 5 + 3 * MM; v++) {
        if (v < nv) {
            const double t = warp_sum(acc[v]);
            if (lane == 0) red[wid][v] = t;
        }
    }
    __syncthreads();
    for (int v = tid; v < nv; v += kAiaThreads) {
        double t = 0;
        for (int w = 0; w < kAiaThreads / 32; w++) t += red[w][v];
        part[(size_t)blockIdx.x * nv + v] = t;
    }
}

// One block: reduce the partials in a fixed order, solve A2 y = b for every
// frame (Cholesky, as LAPACKE_dposv at AIA/aia_cpu.cpp:235), update deltas.
// The convergence measure is max_i |delta_i - old_i| (AIA_CUDAF,
// AIA/aia_cpu.cpp:249-263), or with rel != 0 the change of the shifts
// relative to the first, max_i |(delta_i - delta_0) - (old_i - old_0)|
// (AIA_CUDAF_YC2, AIA/aia_cudaf_v2.cu:665-677), which does not see the
// common rotation the two steps leave free.
__global__ void aia_solve_kernel(const double *__restrict__ part, int nblocks, int M, int N,
                                 double *__restrict__ state, int *__restrict__ done, int max_iter, double max_err,
                                 int rel)
{
    if (*done) return;
    __shared__ double tot[5 + 3 * kAiaMaxM];
    const int nv = 5 + 3 * M;
    for (int v = threadIdx.x; v < nv; v += blockDim.x) {
        double t = 0;
        for (int b = 0; b < nblocks; b++) t += part[(size_t)b * nv + v];
        tot[v] = t;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    const double A[3][3] = {{(double)N, tot[0], tot[2]}, {tot[0], tot[1], tot[3]}, {tot[2], tot[3], tot[4]}};
    double U[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int j = 0; j < 3; j++) {
        double s = A[j][j];
        for (int k = 0; k < j; k++) s -= U[k][j] * U[k][j];
        if (!(s > 0)) {
            state[2 * M + 2] = (double)GLSU_ERR_NOT_POSDEF;
            *done = 1;
            return;
        }
        U[j][j] = sqrt(s);
        for (int i = j + 1; i < 3; i++) {
            double t = A[j][i];
            for (int k = 0; k < j; k++) t -= U[k][j] * U[k][i];
            U[j][i] = t / U[j][j];
        }
    }
    double err = 0, new0 = 0;
    const double old0 = state[0];
    for (int m = 0; m < M; m++) {
        double b[3] = {tot[5 + 3 * m], tot[6 + 3 * m], tot[7 + 3 * m]};
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
        const double dn = atan2(-b[2], b[1]);
        if (m == 0) new0 = dn;
        const double e = rel ? fabs((dn - new0) - (state[m] - old0)) : fabs(dn - state[m]);
        err = e > err ? e : err;
        state[M + m] = state[m];
        state[m] = dn;
    }
    const double it = state[2 * M + 1] + 1;
    state[2 * M + 1] = it;
    state[2 * M] = err;
    if (!(err > max_err) || it >= max_iter) *done = 1;
}

// Normalise the deltas relative to the first one (AIA/aia_cpu.cpp:95-99).
__global__ void aia_norm_kernel(double *__restrict__ state, int M)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double d0 = state[0];
        for (int i = M - 1; i >= 0; i--) {
            const double v = state[i] - d0;
            state[i] = atan2(sin(v), cos(v));
        }
    }
}

template <typename IMG>
static int pass_t(const AiaDev &a, const void *d_frames, int final_pass, float *d_phi, cudaStream_t s)
{
    const IMG *f = (const IMG *)d_frames;
#define GLSU_AIA(MMV)                                                                                       \
    aia_pass_kernel<IMG, MMV><<<a.nblocks, kAiaThreads, 0, s>>>(f, a.M, a.N, a.d_state, a.d_done, a.d_part, \
                                                                final_pass, d_phi)
    if (a.M <= 4) GLSU_AIA(4);
    else if (a.M <= 8) GLSU_AIA(8);
    else if (a.M <= 16) GLSU_AIA(16);
    else GLSU_AIA(32);
#undef GLSU_AIA
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

int aia_launch_pass(const AiaDev &a, int img_type, const void *d_frames, int final_pass, float *d_phi,
                    cudaStream_t s)
{
    if (img_type == GLSU_U8) return pass_t<uint8_t>(a, d_frames, final_pass, d_phi, s);
    if (img_type == GLSU_F32) return pass_t<float>(a, d_frames, final_pass, d_phi, s);
    return fail(GLSU_ERR_INVALID, "AIA frames must be GLSU_U8 or GLSU_F32");
}

int aia_launch_solve(const AiaDev &a, int max_iter, double max_err, cudaStream_t s)
{
    aia_solve_kernel<<<1, 128, 0, s>>>(a.d_part, a.nblocks, a.M, a.N, a.d_state, a.d_done, max_iter, max_err,
                                       a.err_mode == GLSU_AIA_ERR_RELATIVE ? 1 : 0);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

int aia_launch_init(const AiaDev &a, const double *h_deltas, cudaStream_t s)
{
    GLSU_CUDA_TRY(cudaMemcpyAsync(a.d_state, h_deltas, sizeof(double) * a.M, cudaMemcpyHostToDevice, s));
    GLSU_CUDA_TRY(cudaMemsetAsync(a.d_state + a.M, 0, sizeof(double) * (a.M + 3), s));
    GLSU_CUDA_TRY(cudaMemsetAsync(a.d_done, 0, sizeof(int), s));
    return GLSU_OK;
}

int aia_launch_finalize(const AiaDev &a, float *d_phi, cudaStream_t s)
{
    (void)d_phi;
    aia_norm_kernel<<<1, 32, 0, s>>>(a.d_state, a.M);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

}  // namespace glsu
