// dpra_kernels.cu -- DPRA per-pixel windowed least squares on sm_103a.
//
// Reference: DPRA/dpra_cpu.cpp:162-230 (CPU) and DPRA/dpra_hybrid.cu:134-205
// with DPRA/dpra_cudaf.cu:9-92 (GPU).  For each pixel the model
//     I = a + (b cos dphi) cos(phi_ref) - (b sin dphi) sin(phi_ref)
// is fitted over the clipped (2r+1)^2 window; the normal equations are
//     [n0   Sc   Ss ] [x1]   [SI ]
//     [Sc   Scc  Scs] [x2] = [SIc]      n0 = (2r+1)^2 even where the window
//     [Ss   Scs  Sss] [x3]   [SIs]      is clipped (the reference's quirk)
// and dphi = atan2(-x3, x2); the kernel writes exp(j dphi).
//
// Numerics: x1 is eliminated (Schur complement) and the remaining 2x2 system
// is formed from window sums of c, s, I shifted by reference values close to
// the window mean, which removes the cancellation that makes the raw-sum
// normal matrix ill-conditioned where phi_ref is locally smooth (for the
// benchmark sequences the 3x3 condition number reaches 1e6-1e10).  The border
// quirk enters as exact correction terms in rho = 1 - cnt/n0.  Because the
// reduced 2x2 system itself has det/trace^2 ~ 1e-3 on most pixels, the sums
// need more than FP32's 24 bits:
//   FP32 form (default, GLSU_LS_FLOAT_FLOAT): float-float sums and solve of
//              regressors rotated to the tile centre (dpra_ls_ff_kernel);
//   FP32 form (GLSU_LS_FP64_SUMS): c, s in FP64 from the FP32 phase, shift =
//              the tile centre's values, FP64 separable box sums and solve;
//   FP64 form: shift = each pixel's own values (non-separable direct sums),
//              the same evaluation the FP64 oracle uses.
// exp(j dphi) is (X, -Y)/hypot(X, Y) with X ~ x2, Y ~ x3 -- the same value
// as cos/sin of the atan2 without evaluating either.
#include <cmath>

#include "dpra_ls_ff.cuh"
#include "glsu_internal.cuh"

namespace glsu {

constexpr int kDpraTX = 32, kDpraTY = 16;  // outputs per CTA (512 threads)

template <typename T> __device__ __forceinline__ void sincos_t(T a, T *s, T *c);
template <> __device__ __forceinline__ void sincos_t<float>(float a, float *s, float *c) { sincosf(a, s, c); }
template <> __device__ __forceinline__ void sincos_t<double>(double a, double *s, double *c) { sincos(a, s, c); }

// Shared tail: Schur-complement solve from sums shifted by (mc, ms, mi).
template <typename T>
__device__ __forceinline__ C2<T> dpra_solve(double Pc, double Ps, double Pi, double Pcc, double Pss, double Pcs,
                                            double Pic, double Pis, double mc, double ms, double mi, double cnt,
                                            double n0)
{
    const double rho = 1.0 - cnt / n0;
    const double a = Pcc - Pc * Pc / n0 + rho * (2 * mc * Pc + cnt * mc * mc);
    const double d = Pss - Ps * Ps / n0 + rho * (2 * ms * Ps + cnt * ms * ms);
    const double b = Pcs - Pc * Ps / n0 + rho * (mc * Ps + ms * Pc + cnt * mc * ms);
    const double p = Pic - Pi * Pc / n0 + rho * (mi * Pc + mc * Pi + cnt * mi * mc);
    const double q = Pis - Pi * Ps / n0 + rho * (mi * Ps + ms * Pi + cnt * mi * ms);
    double X = d * p - b * q;  // x2 * det
    double Y = a * q - b * p;  // x3 * det
    if (a * d - b * b < 0) {
        X = -X;
        Y = -Y;
    }
    const double h = hypot(X, Y);
    C2<T> out;
    if (h > 0) {
        out.x = (T)(X / h);
        out.y = (T)(-Y / h);
    } else {
        out.x = 1;
        out.y = 0;
    }
    return out;
}

// FP32 form (previous formulation, kept for comparison): FP64 products of
// tile-shifted values, separable box sums.
template <typename IMG, int R> struct SepGeom {
    static constexpr int SW = kDpraTX + 2 * R, SH = kDpraTY + 2 * R;
    static constexpr size_t SMEM = sizeof(double) * 8 * ((size_t)SH * SW + (size_t)SH * kDpraTX);
};

template <typename IMG, int R>
__global__ void __launch_bounds__(kDpraTX *kDpraTY)
    dpra_ls_sep_kernel(const IMG *__restrict__ img, const float *__restrict__ phiref, float2 *__restrict__ z, int W,
                       int H)
{
    using G = SepGeom<IMG, R>;
    constexpr int SW = G::SW, SH = G::SH, NE = SH * SW, NH = SH * kDpraTX;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *v = reinterpret_cast<double *>(smem_raw);  // [8][SH][SW]
    double *hs = v + 8 * NE;                           // [8][SH][32]
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kDpraTX + tx;
    const int x0 = blockIdx.x * kDpraTX, y0 = blockIdx.y * kDpraTY;
    // shift: the values at the tile centre (clamped into the image)
    const size_t cid = (size_t)min(y0 + kDpraTY / 2, H - 1) * W + min(x0 + kDpraTX / 2, W - 1);
    double mc, ms;
    sincos((double)phiref[cid], &ms, &mc);
    const double mi = (double)img[cid];
    for (int e = tid; e < NE; e += kDpraTX * kDpraTY) {
        const int r = e / SW, c = e - r * SW;
        const int gy = y0 - R + r, gx = x0 - R + c;
        double dc = 0, ds = 0, di = 0;
        if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
            const size_t id = (size_t)gy * W + gx;
            double sv, cv;
            sincos((double)phiref[id], &sv, &cv);
            dc = cv - mc;
            ds = sv - ms;
            di = (double)img[id] - mi;
        }
        v[0 * NE + e] = dc;
        v[1 * NE + e] = ds;
        v[2 * NE + e] = di;
        v[3 * NE + e] = dc * dc;
        v[4 * NE + e] = ds * ds;
        v[5 * NE + e] = dc * ds;
        v[6 * NE + e] = di * dc;
        v[7 * NE + e] = di * ds;
    }
    __syncthreads();
    for (int e = tid; e < 8 * NH; e += kDpraTX * kDpraTY) {
        const int k = e / NH, rem = e - k * NH, r = rem / kDpraTX, c = rem - r * kDpraTX;
        const double *src = v + k * NE + r * SW + c;
        double acc = 0;
#pragma unroll
        for (int dx = 0; dx <= 2 * R; dx++) acc += src[dx];
        hs[e] = acc;
    }
    __syncthreads();
    const int gx = x0 + tx, gy = y0 + ty;
    if (gx >= W || gy >= H) return;
    double P[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const double *src = hs + k * NH + ty * kDpraTX + tx;
        double acc = 0;
#pragma unroll
        for (int dy = 0; dy <= 2 * R; dy++) acc += src[dy * kDpraTX];
        P[k] = acc;
    }
    const int m0 = max(gy - R, 0), m1 = min(gy + R, H - 1);
    const int n0 = max(gx - R, 0), n1 = min(gx + R, W - 1);
    const double cnt = (double)((m1 - m0 + 1) * (n1 - n0 + 1));
    z[(size_t)gy * W + gx] = dpra_solve<float>(P[0], P[1], P[2], P[3], P[4], P[5], P[6], P[7], mc, ms, mi, cnt,
                                               (double)((2 * R + 1) * (2 * R + 1)));
}

// FP64 form: sums shifted by each pixel's own values (direct, non-separable).
template <typename IMG, int R>
__global__ void __launch_bounds__(kDpraTX *kDpraTY)
    dpra_ls_f64_kernel(const IMG *__restrict__ img, const double *__restrict__ phiref, double2 *__restrict__ z,
                       int W, int H)
{
    constexpr int SW = kDpraTX + 2 * R, SH = kDpraTY + 2 * R;
    __shared__ double sc[SH][SW + 1], ss[SH][SW + 1], si[SH][SW + 1];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kDpraTX + tx;
    const int x0 = blockIdx.x * kDpraTX, y0 = blockIdx.y * kDpraTY;
    for (int e = tid; e < SW * SH; e += kDpraTX * kDpraTY) {
        const int r = e / SW, c = e - r * SW;
        const int gy = y0 - R + r, gx = x0 - R + c;
        double cv = 0, sv = 0, iv = 0;
        if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
            const size_t id = (size_t)gy * W + gx;
            sincos(phiref[id], &sv, &cv);
            iv = (double)img[id];
        }
        sc[r][c] = cv;
        ss[r][c] = sv;
        si[r][c] = iv;
    }
    __syncthreads();
    const int gx = x0 + tx, gy = y0 + ty;
    if (gx >= W || gy >= H) return;
    const int m0 = max(gy - R, 0), m1 = min(gy + R, H - 1);
    const int n0 = max(gx - R, 0), n1 = min(gx + R, W - 1);
    const double mc = sc[ty + R][tx + R], ms = ss[ty + R][tx + R], mi = si[ty + R][tx + R];
    double pc = 0, ps = 0, pi = 0, pcc = 0, pss = 0, pcs = 0, pic = 0, pis = 0;
    for (int m = m0; m <= m1; m++) {
        const int r = m - y0 + R;
        for (int n = n0; n <= n1; n++) {
            const int c = n - x0 + R;
            const double dc = sc[r][c] - mc, ds = ss[r][c] - ms, di = si[r][c] - mi;
            pc += dc;
            ps += ds;
            pi += di;
            pcc += dc * dc;
            pss += ds * ds;
            pcs += dc * ds;
            pic += di * dc;
            pis += di * ds;
        }
    }
    const double cnt = (double)((m1 - m0 + 1) * (n1 - n0 + 1));
    z[(size_t)gy * W + gx] =
        dpra_solve<double>(pc, ps, pi, pcc, pss, pcs, pic, pis, mc, ms, mi, cnt, (double)((2 * R + 1) * (2 * R + 1)));
}

template <typename IMG, int R>
static int launch_sep(const void *d_img, const void *d_phiref, void *d_z, int W, int H, cudaStream_t s)
{
    using G = SepGeom<IMG, R>;
    GLSU_TRY(raise_smem_limit((const void *)dpra_ls_sep_kernel<IMG, R>, (int)G::SMEM));
    dim3 blk(kDpraTX, kDpraTY), grd((W + kDpraTX - 1) / kDpraTX, (H + kDpraTY - 1) / kDpraTY);
    dpra_ls_sep_kernel<IMG, R><<<grd, blk, G::SMEM, s>>>((const IMG *)d_img, (const float *)d_phiref, (float2 *)d_z,
                                                         W, H);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

template <typename IMG, int R>
static int launch_ff(const void *d_img, const void *d_phiref, void *d_z, int W, int H, cudaStream_t s)
{
    return launch_ff_tile<IMG, R, kDpraTX, kDpraTY>(d_img, d_phiref, d_z, W, H, s);
}

template <typename IMG, int R>
static int launch_f64(const void *d_img, const void *d_phiref, void *d_z, int W, int H, cudaStream_t s)
{
    dim3 blk(kDpraTX, kDpraTY), grd((W + kDpraTX - 1) / kDpraTX, (H + kDpraTY - 1) / kDpraTY);
    dpra_ls_f64_kernel<IMG, R><<<grd, blk, 0, s>>>((const IMG *)d_img, (const double *)d_phiref, (double2 *)d_z,
                                                   W, H);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

template <typename IMG>
static int launch_ls_t(int prec, const void *d_img, const void *d_phiref, void *d_z, int W, int H, int r,
                       cudaStream_t s, int method)
{
#define GLSU_LS_CASE(RR)                                                                                     \
    case RR:                                                                                                 \
        if (prec == GLSU_F64) return launch_f64<IMG, RR>(d_img, d_phiref, d_z, W, H, s);                      \
        return method == GLSU_LS_FP64_SUMS ? launch_sep<IMG, RR>(d_img, d_phiref, d_z, W, H, s)              \
                                           : launch_ff<IMG, RR>(d_img, d_phiref, d_z, W, H, s);
    switch (r) {
        GLSU_LS_CASE(1)
        GLSU_LS_CASE(2)
        GLSU_LS_CASE(3)
        GLSU_LS_CASE(4)
        GLSU_LS_CASE(5)
        GLSU_LS_CASE(6)
        GLSU_LS_CASE(7)
        GLSU_LS_CASE(8)
    default: return fail(GLSU_ERR_UNSUPPORTED, "DPRA window radius must be 1..8");
    }
#undef GLSU_LS_CASE
}

int launch_dpra_ls(int prec, int img_type, const void *d_img, const void *d_phiref, void *d_z, int W, int H, int r,
                   cudaStream_t s, int method, int tile)
{
    if (tile != 0 && prec == GLSU_F32 && method == GLSU_LS_FLOAT_FLOAT)
        return launch_dpra_ls_ff_tile(tile, img_type, d_img, d_phiref, d_z, W, H, r, s);
    if (img_type == GLSU_U8) return launch_ls_t<uint8_t>(prec, d_img, d_phiref, d_z, W, H, r, s, method);
    if (img_type == GLSU_F32) return launch_ls_t<float>(prec, d_img, d_phiref, d_z, W, H, r, s, method);
    if (img_type == GLSU_F64 && prec == GLSU_F64)
        return launch_ls_t<double>(prec, d_img, d_phiref, d_z, W, H, r, s, method);
    return fail(GLSU_ERR_INVALID, "unsupported frame type for this precision");
}

// Phase update of a filtered field (used when WFF2 and the update are run
// as separate calls): DPRA/dpra_hybrid.cu:297-315, DPRA/dpra_cpu.cpp:243-249.
template <typename T>
__global__ void dpra_update_kernel(const C2<T> *__restrict__ f, const T *__restrict__ pr, const T *__restrict__ dpr,
                                   T *__restrict__ pc, T *__restrict__ dp, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const C2<T> v = f[i];
        const T t = atan2(v.y, v.x);
        T s, c;
        sincos_t<T>(t + pr[i], &s, &c);
        pc[i] = atan2(s, c);
        dp[i] = dpr ? dpr[i] + t : t;  // null dphi_ref: the wrapped change alone (unwrapping adds it later)
    }
}

int launch_dpra_update(int prec, const void *d_filtered, const void *phiref, const void *dphiref, void *phicurr,
                       void *dphi, int n, cudaStream_t s)
{
    const int blocks = std::min((n + 255) / 256, 152 * 8);
    if (prec == GLSU_F32)
        dpra_update_kernel<float><<<blocks, 256, 0, s>>>((const float2 *)d_filtered, (const float *)phiref,
                                                         (const float *)dphiref, (float *)phicurr, (float *)dphi, n);
    else
        dpra_update_kernel<double><<<blocks, 256, 0, s>>>((const double2 *)d_filtered, (const double *)phiref,
                                                          (const double *)dphiref, (double *)phicurr,
                                                          (double *)dphi, n);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

}  // namespace glsu
