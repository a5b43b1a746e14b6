// noalloc.cu -- WFF2 (FP32) entry point that allocates no device memory.
//
// Its scratch -- the row-filtered and column-swept planes, the phasor
// tables, the threshold, its partial sums and the error word -- lives in one
// file-scope __device__ array of fixed size.  Every GPU that loads this
// library holds that array until the process exits.  All calls share it:
// each call rewrites what it reads before reading it and clears the error
// word, and two calls whose work overlaps on the GPU race on it.
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "glsu_internal.cuh"

namespace glsu {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;  // 64 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 128;
static std::mutex g_noalloc_mu;
static void *g_noalloc_addr[kMaxDevices];

// Device address of the scratch array on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked up
// once per device (with that device current) and cached.
static int noalloc_scratch(void **out)
{
    int dev = 0;
    GLSU_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(GLSU_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress of the no-allocation scratch");
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return GLSU_OK;
}

// Phasor tables e^{-j w x} computed on the device (no host copies), the fixed
// threshold when one is given, and a cleared error word.
__global__ void noalloc_tables_kernel(float2 *__restrict__ ex, int nfx, int exs, double wxl, double wxi,
                                      float2 *__restrict__ ey, int nfy, int eys, double wyl, double wyi,
                                      float *__restrict__ thr, double thr_value, int *__restrict__ err)
{
    const long long nx = (long long)nfx * exs, total = nx + (long long)nfy * eys;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        double s, c;
        if (t < nx) {
            const int i = (int)(t / exs);
            const double x = (double)(t - (long long)i * exs) - kPhasorPad;
            sincos((wxl + (double)i * wxi) * x, &s, &c);
            ex[t] = make_float2((float)c, (float)-s);
        } else {
            const long long u = t - nx;
            const int k = (int)(u / eys);
            const double y = (double)(u - (long long)k * eys) - kPhasorPad;
            sincos((wyl + (double)k * wyi) * y, &s, &c);
            ey[u] = make_float2((float)c, (float)-s);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (thr_value >= 0) *thr = (float)thr_value;
        *err = 0;
    }
}

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace glsu

using namespace glsu;

extern "C" int glsu_wff_run_noalloc(int width, int height, const glsu_wff_params *p, const void *d_f,
                                    void *d_filtered, void *cuda_stream)
{
    if (!d_f || !d_filtered) return fail(GLSU_ERR_INVALID, "null argument");
    glsu_wff_params prm;
    if (p) prm = *p;
    else glsu_wft_default_params(GLSU_WFT_WFF, &prm);
    WffPlan P;
    GLSU_TRY(P.init(GLSU_F32, width, height, prm));

    const size_t exs = (size_t)P.pitch + 2 * kPhasorPad, eys = (size_t)P.H + 2 * kPhasorPad;
    const size_t off_R = 0;
    const size_t off_C = off_R + align256((size_t)P.nfx * P.plane_bytes());
    const size_t off_ex = off_C + align256((size_t)P.nfx * P.plane_bytes());
    const size_t off_ey = off_ex + align256((size_t)P.nfx * exs * sizeof(float2));
    const size_t off_thr = off_ey + align256((size_t)P.nfy * eys * sizeof(float2));
    const size_t off_part = off_thr + 256;
    const size_t off_err = off_part + align256(sizeof(double) * kThrBlocks);
    const size_t total = off_err + 256;
    if (total > kNoAllocScratchBytes) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "glsu_wff_run_noalloc: %dx%d with %dx%d frequencies needs %.1f MiB of scratch; its fixed scratch "
                 "holds %zu MiB (use glsu_wff_create/glsu_wff_run for larger problems)",
                 width, height, P.nfx, P.nfy, total / 1048576.0, kNoAllocScratchBytes >> 20);
        return fail(GLSU_ERR_INVALID, msg);
    }

    void *base = nullptr;
    GLSU_TRY(noalloc_scratch(&base));
    unsigned char *b = static_cast<unsigned char *>(base);
    P.external_scratch = true;
    P.d_R = b + off_R;
    P.d_C = b + off_C;
    P.d_ex = b + off_ex;
    P.d_ey = b + off_ey;
    P.d_thr = b + off_thr;
    P.d_part = reinterpret_cast<double *>(b + off_part);
    P.d_err = reinterpret_cast<int *>(b + off_err);

    cudaStream_t s = (cudaStream_t)cuda_stream;
    const long long entries = (long long)P.nfx * exs + (long long)P.nfy * eys;
    const int blocks = (int)std::min<long long>((entries + 255) / 256, 152 * 4);
    noalloc_tables_kernel<<<blocks, 256, 0, s>>>((float2 *)P.d_ex, P.nfx, (int)exs, prm.wxl, prm.wxi,
                                                 (float2 *)P.d_ey, P.nfy, (int)eys, prm.wyl, prm.wyi,
                                                 (float *)P.d_thr, prm.thr, P.d_err);
    GLSU_CUDA_TRY(cudaGetLastError());
    GLSU_TRY(P.make_tensor_map());
    GLSU_TRY(P.enqueue(s, d_f, d_filtered, 0, nullptr, nullptr, nullptr, nullptr, nullptr));
    return P.check_device_error(s);
}
