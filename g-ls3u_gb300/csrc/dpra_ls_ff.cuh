// dpra_ls_ff.cuh -- the FP32 DPRA least squares in float-float arithmetic
// (see dpra_kernels.cu for the normal equations and the reference lines),
// templated on the output tile so that the tile shape is a tuning knob.
#pragma once

#include "glsu_internal.cuh"

namespace glsu {

// ---------------------------------------------------------------------------
// FP32 form in float-float arithmetic (no FP64 on the FP32 path).
//
// A float-float value is hi + lo with |lo| <= ulp(hi)/2: about 48 bits of
// mantissa from FP32 operations alone (Dekker / Knuth error-free
// transformations: TwoSum, and TwoProduct through fmaf).  On GB300 the FP64
// rate is a small fraction of the FP32 rate, so the window sums and the
// Schur-complement solve, which need more than FP32's 24 bits because the
// normal matrix is ill-conditioned, are formed this way.
//
// The regressors are taken in a frame rotated by the tile centre's phase
// phi_t: with u = phi - phi_t, C = cos u and S = sin u satisfy
//   x2 cos phi + x3 sin phi = x2' C + x3' S,  (x2', x3') = R(phi_t) (x2, x3),
// and C - 1, S are formed in float-float from the exact difference u (no
// cancellation against cos phi_t).  FP32 storage of C - 1 and S is not
// enough: through the least-squares residual their rounding reaches the
// solution amplified by the normal matrix's condition number (up to 1e4-1e6
// here), giving 6.6e-4 rad (256^2) and 1.2e-2 rad (512^2) worst-case errors in
// an FP64 emulation, against 8e-11 / 2.5e-9 with exact regressors.
// ---------------------------------------------------------------------------
struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ ff ff_fast_two_sum(float a, float b)  // |a| >= |b|
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff ff_two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, fmaf(a, b, -p)};
}

__device__ __forceinline__ ff ff_add(ff x, ff y)
{
    ff s = ff_two_sum(x.hi, y.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo));
    return ff_fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ ff ff_neg(ff x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ ff ff_sub(ff x, ff y) { return ff_add(x, ff_neg(y)); }

__device__ __forceinline__ ff ff_mul(ff x, ff y)
{
    ff p = ff_two_prod(x.hi, y.hi);
    p.lo = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, p.lo));
    return ff_fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ ff ff_from(float a) { return {a, 0.f}; }

__device__ __forceinline__ ff ff_mul_f(ff x, float y)
{
    ff p = ff_two_prod(x.hi, y);
    p.lo = fmaf(x.lo, y, p.lo);
    return ff_fast_two_sum(p.hi, p.lo);
}

// Float-float constants below are the splits hi = fl32(c), lo = fl32(c - hi)
// of pi/2 and of the Taylor coefficients +-1/n!.

// sin(u) and cos(u) - 1 in float-float for a float-float angle u with
// |u| <= 2 pi.  Reduction u = k pi/2 + r with |r| <= pi/4 (pi/2 held as a
// float-float constant, k small, so k pi/2 is formed exactly by TwoProduct),
// then the Taylor series of sin r and cos r - 1 in Horner form on r^2; for
// |r| <= pi/4 the first omitted terms are below 5e-17.  cos u - 1 keeps its
// relative accuracy near u = 0 because its series is summed without the 1.
__device__ __forceinline__ void ff_sincos_m1(ff u, ff *sn, ff *cm1)
{
    const ff pio2 = ff{1.5707963705062866f, -4.371138828673793e-08f};
    const float k = rintf(__fmul_rn(u.hi, 0.63661977236758134f));
    const ff kp = ff_add(ff_two_prod(k, pio2.hi), ff_from(__fmul_rn(k, pio2.lo)));
    const ff r = ff_sub(u, kp);
    const ff r2 = ff_mul(r, r);
    // sin r = r (1 - r^2/3! + r^4/5! - ... - r^14/15!)
    ff ps = ff{-7.647163609812713e-13f, -1.2200710471178288e-20f};
    ps = ff_add(ff_mul(ps, r2), ff{1.6059044372074283e-10f, -5.352526511562726e-18f});
    ps = ff_add(ff_mul(ps, r2), ff{-2.5052107943679403e-08f, -4.4176230446483665e-16f});
    ps = ff_add(ff_mul(ps, r2), ff{2.7557318844628753e-06f, 3.793571224297229e-14f});
    ps = ff_add(ff_mul(ps, r2), ff{-0.00019841270113829523f, 2.725596874933456e-12f});
    ps = ff_add(ff_mul(ps, r2), ff{0.008333333767950535f, -4.34617203337595e-10f});
    ps = ff_add(ff_mul(ps, r2), ff{-0.1666666716337204f, 4.967053879312289e-09f});
    const ff sr = ff_add(r, ff_mul(ff_mul(ps, r2), r));
    // cos r - 1 = r^2 (-1/2! + r^2/4! - ... + r^14/16!)
    ff pc = ff{4.7794772561329454e-14f, 7.62544404448643e-22f};
    pc = ff_add(ff_mul(pc, r2), ff{-1.147074536050896e-11f, -2.372207689231238e-19f});
    pc = ff_add(ff_mul(pc, r2), ff{2.0876755879584152e-09f, 1.1082839809204342e-16f});
    pc = ff_add(ff_mul(pc, r2), ff{-2.755731998149713e-07f, 7.575112209051195e-15f});
    pc = ff_add(ff_mul(pc, r2), ff{2.4801587642286904e-05f, -3.40699609366682e-13f});
    pc = ff_add(ff_mul(pc, r2), ff{-0.0013888889225199819f, 3.3631094437103215e-11f});
    pc = ff_add(ff_mul(pc, r2), ff{0.0416666679084301f, -1.2417634698280722e-09f});
    pc = ff_add(ff_mul(pc, r2), ff{-0.5f, 0.0f});
    const ff cr1 = ff_mul(pc, r2);
    const ff one = {1.f, 0.f};
    const int q = ((int)k) & 3;
    if (q == 0) {
        *sn = sr;
        *cm1 = cr1;
    } else if (q == 1) {  // sin u = cos r, cos u = -sin r
        *sn = ff_add(cr1, one);
        *cm1 = ff_sub(ff_neg(sr), one);
    } else if (q == 2) {  // sin u = -sin r, cos u = -cos r
        *sn = ff_neg(sr);
        *cm1 = ff_sub(ff_neg(cr1), ff_from(2.f));
    } else {  // sin u = -cos r, cos u = sin r
        *sn = ff_neg(ff_add(cr1, one));
        *cm1 = ff_sub(sr, one);
    }
}

// 1/n as float-float (n a small positive integer)
__device__ __forceinline__ ff ff_recip(float n)
{
    const float r = __frcp_rn(n);
    const float e = fmaf(-n, r, 1.0f);  // 1 - n r, exact
    return ff_fast_two_sum(r, __fmul_rn(e, r));
}

// Schur-complement solve in float-float for shifts (mc, ms, mi) = (1, 0, mi)
// of the rotated regressors; returns (X, Y) ~ (x2', x3') * det.
__device__ __forceinline__ void dpra_solve_ff(const ff *P, float mi, float cnt, float n0, float *X, float *Y)
{
    const ff inv = ff_recip(n0);
    const ff rho = ff_mul(ff_from(n0 - cnt), inv);  // 1 - cnt/n0, n0 - cnt exact
    const ff Pc = P[0], Ps = P[1], Pi = P[2], Pcc = P[3], Pss = P[4], Pcs = P[5], Pic = P[6], Pis = P[7];
    const ff m = ff_from(mi);
    // a = Pcc - Pc^2/n0 + rho (2 Pc + cnt)
    const ff a = ff_add(ff_sub(Pcc, ff_mul(ff_mul(Pc, Pc), inv)), ff_mul(rho, ff_add(ff_add(Pc, Pc), ff_from(cnt))));
    // d = Pss - Ps^2/n0
    const ff d = ff_sub(Pss, ff_mul(ff_mul(Ps, Ps), inv));
    // b = Pcs - Pc Ps/n0 + rho Ps
    const ff b = ff_add(ff_sub(Pcs, ff_mul(ff_mul(Pc, Ps), inv)), ff_mul(rho, Ps));
    // p = Pic - Pi Pc/n0 + rho (mi Pc + Pi + cnt mi)
    const ff p = ff_add(ff_sub(Pic, ff_mul(ff_mul(Pi, Pc), inv)),
                        ff_mul(rho, ff_add(ff_add(ff_mul(m, Pc), Pi), ff_two_prod(cnt, mi))));
    // q = Pis - Pi Ps/n0 + rho mi Ps
    const ff q = ff_add(ff_sub(Pis, ff_mul(ff_mul(Pi, Ps), inv)), ff_mul(rho, ff_mul(m, Ps)));
    ff x = ff_sub(ff_mul(d, p), ff_mul(b, q));
    ff y = ff_sub(ff_mul(a, q), ff_mul(b, p));
    const ff det = ff_sub(ff_mul(a, d), ff_mul(b, b));
    float xs = __fadd_rn(x.hi, x.lo), ys = __fadd_rn(y.hi, y.lo);
    if (det.hi < 0) {
        xs = -xs;
        ys = -ys;
    }
    *X = xs;
    *Y = ys;
}

// Dynamic shared memory of a TX x TY output tile at radius r: per halo
// element 8 float-float values (C-1, S, I-I_t and the five products), per
// horizontal sum 8 float-float; odd row strides (in float-float elements):
// the running-sum passes walk rows with consecutive threads, which then meet
// distinct bank pairs.
__host__ __device__ constexpr size_t ff_ls_smem_bytes(int tx, int ty, int r)
{
    return sizeof(float) * 2 * (8 * (size_t)((tx + 2 * r) | 1) * (ty + 2 * r) + 8 * (size_t)(ty + 2 * r) * (tx + 1));
}

template <int R, int TX, int TY> struct FfGeom {
    static constexpr int SW = TX + 2 * R, SH = TY + 2 * R;
    static constexpr int SWP = SW | 1, HSP = TX + 1;
    static constexpr int NE = SWP * SH, NH = SH * HSP;
    static constexpr size_t SMEM = ff_ls_smem_bytes(TX, TY, R);
    static_assert(SMEM == sizeof(ff) * (8 * (size_t)NE + 8 * (size_t)NH), "shared-memory layout");
    static_assert(NE >= TX * TY, "the vertical sums reuse the product buffer");
    static_assert(TX % 8 == 0 && TY % 8 == 0, "running sums over segments of 8 outputs");
};

template <typename IMG, int R, int TX, int TY>
__global__ void __launch_bounds__(TX *TY)
    dpra_ls_ff_kernel(const IMG *__restrict__ img, const float *__restrict__ phiref, float2 *__restrict__ z, int W,
                      int H)
{
    using G = FfGeom<R, TX, TY>;
    constexpr int SW = G::SW, SWP = G::SWP, HSP = G::HSP, NE = G::NE, NH = G::NH;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ff *pr = reinterpret_cast<ff *>(smem_raw);  // [8][SH][SWP]: C-1, S, I-I_t, CC, SS, CS, IC, IS
    ff *hs = pr + 8 * NE;                       // [8][SH][HSP] horizontal sums
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const size_t cid = (size_t)min(y0 + TY / 2, H - 1) * W + min(x0 + TX / 2, W - 1);
    const float phit = phiref[cid];
    const float mi = (float)img[cid];
    for (int e0 = tid; e0 < G::SH * SW; e0 += TX * TY) {
        const int r = e0 / SW, c = e0 - r * SW, e = r * SWP + c;
        const int gy = y0 - R + r, gx = x0 - R + c;
        ff dc = {0.f, 0.f}, ds = {0.f, 0.f}, di = {0.f, 0.f};
        if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
            const size_t id = (size_t)gy * W + gx;
            ff_sincos_m1(ff_two_sum(phiref[id], -phit), &ds, &dc);  // u = phi - phi_t, exact
            di = ff_two_sum((float)img[id], -mi);
        }
        pr[e] = dc;
        pr[NE + e] = ds;
        pr[2 * NE + e] = di;
        pr[3 * NE + e] = ff_mul(dc, dc);
        pr[4 * NE + e] = ff_mul(ds, ds);
        pr[5 * NE + e] = ff_mul(dc, ds);
        pr[6 * NE + e] = ff_mul(di, dc);
        pr[7 * NE + e] = ff_mul(di, ds);
    }
    __syncthreads();
    // box sums as running sums over segments of kSeg outputs: the first sum
    // of a segment in full, each next one by adding the entering value and
    // subtracting the leaving one (about 2 float-float additions per output
    // instead of 2R + 1); horizontal sums of every halo row, then vertical
    // sums into ps (the products are not read again)
    constexpr int kSeg = 8;
    constexpr int NSX = TX / kSeg, NSY = TY / kSeg;
    for (int e = tid; e < 8 * G::SH * NSX; e += TX * TY) {
        const int r = e % G::SH, rest = e / G::SH, sg = rest % NSX, k = rest / NSX;
        const ff *src = pr + k * NE + r * SWP + sg * kSeg;
        ff *dst = hs + k * NH + r * HSP + sg * kSeg;
        ff acc = src[0];
#pragma unroll
        for (int dx = 1; dx <= 2 * R; dx++) acc = ff_add(acc, src[dx]);
        dst[0] = acc;
#pragma unroll
        for (int c = 1; c < kSeg; c++) {
            acc = ff_sub(ff_add(acc, src[c + 2 * R]), src[c - 1]);
            dst[c] = acc;
        }
    }
    __syncthreads();
    ff *ps = pr;  // [8][TY][TX]
    for (int e = tid; e < 8 * TX * NSY; e += TX * TY) {
        const int c = e % TX, rest = e / TX, sg = rest % NSY, k = rest / NSY;
        const ff *src = hs + k * NH + sg * kSeg * HSP + c;
        ff *dst = ps + (k * TY + sg * kSeg) * TX + c;
        ff acc = src[0];
#pragma unroll
        for (int dy = 1; dy <= 2 * R; dy++) acc = ff_add(acc, src[dy * HSP]);
        dst[0] = acc;
#pragma unroll
        for (int y = 1; y < kSeg; y++) {
            acc = ff_sub(ff_add(acc, src[(y + 2 * R) * HSP]), src[(y - 1) * HSP]);
            dst[y * TX] = acc;
        }
    }
    __syncthreads();
    const int gx = x0 + tx, gy = y0 + ty;
    if (gx >= W || gy >= H) return;
    ff P[8];
#pragma unroll
    for (int k = 0; k < 8; k++) P[k] = ps[(k * TY + ty) * TX + tx];
    const int m0 = max(gy - R, 0), m1 = min(gy + R, H - 1);
    const int n0 = max(gx - R, 0), n1 = min(gx + R, W - 1);
    const float cnt = (float)((m1 - m0 + 1) * (n1 - n0 + 1));
    float X, Y;
    dpra_solve_ff(P, mi, cnt, (float)((2 * R + 1) * (2 * R + 1)), &X, &Y);
    // back from the rotated frame: (x2, x3) = R(-phi_t) (x2', x3')
    float st, ct;
    sincosf(phit, &st, &ct);
    const float x2 = ct * X - st * Y, x3 = st * X + ct * Y;
    const float h = hypotf(x2, x3);
    z[(size_t)gy * W + gx] = h > 0.f ? make_float2(x2 / h, -x3 / h) : make_float2(1.f, 0.f);
}


// Launch the float-float LS with a TX x TY output tile (TX x TY threads).
template <typename IMG, int R, int TX, int TY>
static int launch_ff_tile(const void *d_img, const void *d_phiref, void *d_z, int W, int H, cudaStream_t s)
{
    using G = FfGeom<R, TX, TY>;
    GLSU_TRY(raise_smem_limit((const void *)dpra_ls_ff_kernel<IMG, R, TX, TY>, (int)G::SMEM));
    dim3 blk(TX, TY), grd((W + TX - 1) / TX, (H + TY - 1) / TY);
    dpra_ls_ff_kernel<IMG, R, TX, TY><<<grd, blk, G::SMEM, s>>>((const IMG *)d_img, (const float *)d_phiref,
                                                                (float2 *)d_z, W, H);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

// Tile variants other than the default, compiled in dpra_ls_tiles.cu:
// tile 1 = 32 x 8, tile 2 = 32 x 32 outputs per CTA.
int launch_dpra_ls_ff_tile(int tile, int img_type, const void *d_img, const void *d_phiref, void *d_z, int W, int H,
                           int r, cudaStream_t s);

}  // namespace glsu
