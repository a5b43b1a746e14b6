// wff_common.cuh -- small helpers shared by the WFF2 and WFR2 sweep kernels
// (wff_kernels.cu, wfr_kernels.cu): window taps passed as kernel parameters,
// complex construction and the real-tap complex FMA.
#pragma once

#include "glsu_internal.cuh"

namespace glsu {

template <typename T, int S> struct Taps {
    T g[2 * S + 1];
};

template <typename T> __device__ __forceinline__ C2<T> mk(T x, T y)
{
    C2<T> r;
    r.x = x;
    r.y = y;
    return r;
}

// acc += g * v for a real tap g and a complex v: two scalar FMAs, whose tap
// operand comes straight from the kernel-parameter bank.  (The packed
// __ffma2_rn needs {g, g} in a register pair; with 2S+1 = 61 taps that cost a
// move per FMA and made the 1024^2 column sweep 2.9x slower, 16.2 vs 5.5 ms.)
__device__ __forceinline__ void cfma(float2 &acc, float g, float2 v)
{
    acc.x = fmaf(g, v.x, acc.x);
    acc.y = fmaf(g, v.y, acc.y);
}
__device__ __forceinline__ void cfma(double2 &acc, double g, double2 v)
{
    acc.x = fma(g, v.x, acc.x);
    acc.y = fma(g, v.y, acc.y);
}

// Taps of the instantiated half size S from the true half size strue
// (zero beyond it), scaled by mul.
template <typename T, int S> inline Taps<T, S> make_taps(const double *g, int strue, double mul)
{
    Taps<T, S> t;
    for (int m = 0; m <= 2 * S; m++) {
        const int k = m - S;  // offset
        t.g[m] = (k >= -strue && k <= strue) ? (T)(g[k + strue] * mul) : (T)0;
    }
    return t;
}

}  // namespace glsu
