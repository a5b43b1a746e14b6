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
// is formed from sums of values shifted by the centre pixel's c, s, I, which
// removes the cancellation that makes the raw-sum normal matrix
// ill-conditioned where phi_ref is locally flat.  The border quirk enters as
// exact correction terms in rho = 1 - cnt/n0.  The shifted sums use Kahan
// compensation in the FP32 form; the 2x2 solve runs in FP64 in both forms.
// exp(j dphi) is (X, -Y)/hypot(X, Y) with X ~ x2, Y ~ x3 -- the same value
// as cos/sin of the atan2 without evaluating either.
#include <cmath>

#include "glsu_internal.cuh"

namespace glsu {

constexpr int kDpraTX = 32, kDpraTY = 16;  // outputs per CTA (512 threads)

template <typename T> struct Kahan {
    T s = 0, c = 0;
    __device__ __forceinline__ void add(T v)
    {
        const T y = v - c;
        const T t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

template <typename T> __device__ __forceinline__ void sincos_t(T a, T *s, T *c);
template <> __device__ __forceinline__ void sincos_t<float>(float a, float *s, float *c) { sincosf(a, s, c); }
template <> __device__ __forceinline__ void sincos_t<double>(double a, double *s, double *c) { sincos(a, s, c); }

template <typename IMG> __device__ __forceinline__ double load_img(const IMG *p, size_t i) { return (double)p[i]; }

template <typename T, typename IMG, int R>
__global__ void __launch_bounds__(kDpraTX *kDpraTY)
    dpra_ls_kernel(const IMG *__restrict__ img, const T *__restrict__ phiref, C2<T> *__restrict__ z, int W, int H)
{
    constexpr int SW = kDpraTX + 2 * R, SH = kDpraTY + 2 * R;
    __shared__ T sc[SH][SW + 1], ss[SH][SW + 1], si[SH][SW + 1];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kDpraTX + tx;
    const int x0 = blockIdx.x * kDpraTX, y0 = blockIdx.y * kDpraTY;
    for (int e = tid; e < SW * SH; e += kDpraTX * kDpraTY) {
        const int r = e / SW, c = e - r * SW;
        const int gy = y0 - R + r, gx = x0 - R + c;
        T cv = 0, sv = 0, iv = 0;
        if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
            const size_t id = (size_t)gy * W + gx;
            sincos_t<T>(phiref[id], &sv, &cv);
            iv = (T)img[id];
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
    const T mc = sc[ty + R][tx + R], ms = ss[ty + R][tx + R], mi = si[ty + R][tx + R];
    Kahan<T> pc, ps, pi, pcc, pss, pcs, pic, pis;
    for (int m = m0; m <= m1; m++) {
        const int r = m - y0 + R;
        for (int n = n0; n <= n1; n++) {
            const int c = n - x0 + R;
            const T dc = sc[r][c] - mc, ds = ss[r][c] - ms, di = si[r][c] - mi;
            pc.add(dc);
            ps.add(ds);
            pi.add(di);
            pcc.add(dc * dc);
            pss.add(ds * ds);
            pcs.add(dc * ds);
            pic.add(di * dc);
            pis.add(di * ds);
        }
    }
    const double cnt = (double)((m1 - m0 + 1) * (n1 - n0 + 1));
    const double n0d = (double)((2 * R + 1) * (2 * R + 1));
    const double rho = 1.0 - cnt / n0d;
    const double Pc = pc.s, Ps = ps.s, Pi = pi.s;
    const double Mc = mc, Ms = ms, Mi = mi;
    const double a = (double)pcc.s - Pc * Pc / n0d + rho * (2 * Mc * Pc + cnt * Mc * Mc);
    const double d = (double)pss.s - Ps * Ps / n0d + rho * (2 * Ms * Ps + cnt * Ms * Ms);
    const double b = (double)pcs.s - Pc * Ps / n0d + rho * (Mc * Ps + Ms * Pc + cnt * Mc * Ms);
    const double p = (double)pic.s - Pi * Pc / n0d + rho * (Mi * Pc + Mc * Pi + cnt * Mi * Mc);
    const double q = (double)pis.s - Pi * Ps / n0d + rho * (Mi * Ps + Ms * Pi + cnt * Mi * Ms);
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
    z[(size_t)gy * W + gx] = out;
}

template <typename T, typename IMG>
static int launch_ls_t(const void *d_img, const void *d_phiref, void *d_z, int W, int H, int r, cudaStream_t s)
{
    dim3 blk(kDpraTX, kDpraTY), grd((W + kDpraTX - 1) / kDpraTX, (H + kDpraTY - 1) / kDpraTY);
    const IMG *im = (const IMG *)d_img;
    const T *ph = (const T *)d_phiref;
    C2<T> *zz = (C2<T> *)d_z;
    switch (r) {
    case 1: dpra_ls_kernel<T, IMG, 1><<<grd, blk, 0, s>>>(im, ph, zz, W, H); break;
    case 2: dpra_ls_kernel<T, IMG, 2><<<grd, blk, 0, s>>>(im, ph, zz, W, H); break;
    case 3: dpra_ls_kernel<T, IMG, 3><<<grd, blk, 0, s>>>(im, ph, zz, W, H); break;
    case 4: dpra_ls_kernel<T, IMG, 4><<<grd, blk, 0, s>>>(im, ph, zz, W, H); break;
    case 5: dpra_ls_kernel<T, IMG, 5><<<grd, blk, 0, s>>>(im, ph, zz, W, H); break;
    case 6: dpra_ls_kernel<T, IMG, 6><<<grd, blk, 0, s>>>(im, ph, zz, W, H); break;
    case 7: dpra_ls_kernel<T, IMG, 7><<<grd, blk, 0, s>>>(im, ph, zz, W, H); break;
    case 8: dpra_ls_kernel<T, IMG, 8><<<grd, blk, 0, s>>>(im, ph, zz, W, H); break;
    default: return fail(GLSU_ERR_UNSUPPORTED, "DPRA window radius must be 1..8");
    }
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

int launch_dpra_ls(int prec, int img_type, const void *d_img, const void *d_phiref, void *d_z, int W, int H, int r,
                   cudaStream_t s)
{
    if (prec == GLSU_F32) {
        if (img_type == GLSU_U8) return launch_ls_t<float, uint8_t>(d_img, d_phiref, d_z, W, H, r, s);
        if (img_type == GLSU_F32) return launch_ls_t<float, float>(d_img, d_phiref, d_z, W, H, r, s);
    } else {
        if (img_type == GLSU_U8) return launch_ls_t<double, uint8_t>(d_img, d_phiref, d_z, W, H, r, s);
        if (img_type == GLSU_F32) return launch_ls_t<double, float>(d_img, d_phiref, d_z, W, H, r, s);
        if (img_type == GLSU_F64) return launch_ls_t<double, double>(d_img, d_phiref, d_z, W, H, r, s);
    }
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
        dp[i] = dpr[i] + t;
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
