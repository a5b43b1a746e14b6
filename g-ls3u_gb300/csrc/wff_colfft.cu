// wff_colfft.cu -- host side of the WFF2 FFT column sweep (FP32 form): the
// transform length and CTA width of a plan, its tables, the launch, and the
// column-sweep autotuner.  The kernels are in wff_colfft.cuh, compiled per
// transform length in wff_colfft_k{1,2,3}.cu.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "wff_colfft_plans.cuh"

namespace glsu {

namespace colfft {

bool len_info(int L, LenInfo *out)
{
#define GLSU_LEN(LEN, PLAN, NC0)                                                    \
    case LEN:                                                                       \
        *out = LenInfo{LEN, PLAN::T, PLAN::NP, NC0, smem_per_column<PLAN>()};       \
        return true;
    switch (L) {
        GLSU_LEN(256, P256, 4)
        GLSU_LEN(384, P384, 8)
        GLSU_LEN(512, P512, 4)
        GLSU_LEN(640, P640, 8)
        GLSU_LEN(768, P768, 4)
        GLSU_LEN(1024, P1024, 4)
        GLSU_LEN(1280, P1280, 4)
        GLSU_LEN(1536, P1536, 2)
        GLSU_LEN(2048, P2048, 2)
        GLSU_LEN(2560, P2560, 2)
        GLSU_LEN(3072, P3072, 1)
        GLSU_LEN(4096, P4096, 1)
    default: return false;
    }
#undef GLSU_LEN
}

}  // namespace colfft

// Compiled transform lengths >= need, ascending; at most n of them.
static int length_candidates(int need, int *out, int n)
{
    int k = 0;
    for (int i = 0; i < colfft::kNumLengths && k < n; i++)
        if (colfft::kLengths[i] >= need) out[k++] = colfft::kLengths[i];
    return k;
}

// CTA widths (columns per CTA) compiled for length L: the default and twice it.
static bool ncol_ok(int L, int nc, int pitch)
{
    colfft::LenInfo li;
    if (!colfft::len_info(L, &li)) return false;
    if (nc != li.ncol_default && nc != 2 * li.ncol_default) return false;
    return li.T * nc <= 512 && (size_t)nc * li.smem_col <= 227 * 1024 && pitch % nc == 0;
}

int WffPlan::init_colfft()
{
    if (prec != GLSU_F32) return GLSU_OK;
    int L;
    if (length_candidates(H + 2 * sy, &L, 1) < 1) return GLSU_OK;  // taller than the longest plan: direct kernel
    return build_colfft(L);
}

// Tables of the FFT sweep for transform length L (replacing any others),
// with the default CTA width: H_k = DFT of h_k(m) = gy(m) e^{j wy_k m},
// m in [-sy, sy] placed circularly, and the twiddles e^{-2 pi i t / L},
// both computed in FP64.
int WffPlan::build_colfft(int L)
{
    colfft::LenInfo li;
    if (prec != GLSU_F32 || L < H + 2 * sy || !colfft::len_info(L, &li))
        return fail(GLSU_ERR_UNSUPPORTED, "no compiled FFT plan of that length for this handle");
    release_colfft();
    std::vector<float> kh(2 * (size_t)nfy * L), tw(2 * (size_t)L);
    for (int k = 0; k < nfy; k++) {
        const double wy = this->p.wyl + (double)k * this->p.wyi;
        for (int w = 0; w < L; w++) {
            double re = 0, im = 0;
            for (int m = -sy; m <= sy; m++) {
                const double ang = wy * m - 2.0 * M_PI * (double)w * (double)m / (double)L;
                re += gy[m + sy] * std::cos(ang);
                im += gy[m + sy] * std::sin(ang);
            }
            kh[2 * ((size_t)k * L + w)] = (float)re;
            kh[2 * ((size_t)k * L + w) + 1] = (float)im;
        }
    }
    for (int t = 0; t < L; t++) {
        tw[2 * t] = (float)std::cos(-2.0 * M_PI * t / L);
        tw[2 * t + 1] = (float)std::sin(-2.0 * M_PI * t / L);
    }
    if (cudaMalloc(&d_khat, kh.size() * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&d_tw, tw.size() * sizeof(float)) != cudaSuccess) {
        release_colfft();
        return fail(GLSU_ERR_ALLOC, "cudaMalloc of the column FFT tables failed");
    }
    GLSU_CUDA_TRY(cudaMemcpy(d_khat, kh.data(), kh.size() * sizeof(float), cudaMemcpyHostToDevice));
    GLSU_CUDA_TRY(cudaMemcpy(d_tw, tw.data(), tw.size() * sizeof(float), cudaMemcpyHostToDevice));
    fft_L = L;
    fft_nst = li.passes;
    return set_fft_plan(li.ncol_default, 0);
}

int fft_length_candidates(const WffPlan &P, int *out, int n)
{
    if (P.prec != GLSU_F32 || P.fft_L == 0) return 0;
    return length_candidates(P.H + 2 * P.sy, out, n);
}

// Plan variant: nc columns per CTA (the length's default or twice it);
// radix order 0 only (each length has one compiled radix sequence).
int WffPlan::set_fft_plan(int nc, int order)
{
    if (fft_L == 0) return fail(GLSU_ERR_UNSUPPORTED, "no shared-memory FFT plan for this handle");
    if (order != 0 || !ncol_ok(fft_L, nc, pitch))
        return fail(GLSU_ERR_UNSUPPORTED, "FFT plan variant not compiled for this transform length");
    fft_nc = nc;
    fft_order = order;
    return GLSU_OK;
}

void WffPlan::release_colfft()
{
    cudaFree(d_khat);
    cudaFree(d_tw);
    d_khat = d_tw = nullptr;
    fft_L = 0;
}

int launch_colfft(const WffPlan &P, cudaStream_t s)
{
    const int ngroups = P.pitch / P.fft_nc;
    int grid_x = ngroups;
    const int2 *list = nullptr;
    const int *count = nullptr;
    if (P.mask.flags) {
        // tile-masked run (the surrogate's per-tile fallback): the column
        // groups whose columns, grown by sx, meet a flagged tile; all rows,
        // since a column's transform spans them.  Each column is computed as
        // in the full frame, so its outputs are the same bits.
        if (!P.d_list) return fail(GLSU_ERR_INVALID, "tile-masked run without a tile list buffer");
        TileMask m = P.mask;
        m.my = 0;
        m.mx = P.sx;
        GLSU_TRY(launch_mask_list(m, ngroups, 1, P.H, P.fft_nc, P.d_list, P.d_list_count, s));
        list = P.d_list;
        count = P.d_list_count;
        grid_x = std::max(1, std::min(ngroups, (2 * device_sm_count() + P.nfx - 1) / P.nfx));
    }
    int rc = colfft::launch_len_small(P.fft_L, P.fft_nc, P, s, list, count, grid_x);
    if (rc == GLSU_ERR_UNSUPPORTED) rc = colfft::launch_len_mid(P.fft_L, P.fft_nc, P, s, list, count, grid_x);
    if (rc == GLSU_ERR_UNSUPPORTED) rc = colfft::launch_len_large(P.fft_L, P.fft_nc, P, s, list, count, grid_x);
    if (rc == GLSU_ERR_UNSUPPORTED) return fail(GLSU_ERR_UNSUPPORTED, "no compiled FFT plan for this length");
    return rc;
}

// The FFT column sweep of n plans that share one transform length, as one
// persistent launch (per 128 plans) over their (plan, plane, column group)
// work list, at the length's default CTA width.  Each column is computed
// exactly as launch_colfft computes it, so the outputs are the same bits.
int launch_colfft_batch(const WffPlan *const *plans, int n, cudaStream_t s)
{
    if (n <= 0) return GLSU_OK;
    const int L = plans[0]->fft_L;
    colfft::LenInfo li;
    if (!colfft::len_info(L, &li)) return fail(GLSU_ERR_UNSUPPORTED, "no compiled FFT plan for this length");
    const int nc = li.ncol_default;
    static thread_local colfft::BatchTable tab;
    for (int i0 = 0; i0 < n; i0 += colfft::kMaxBatchSeqs) {
        const int m = std::min(n - i0, colfft::kMaxBatchSeqs);
        int nitems = 0;
        for (int k = 0; k < m; k++) {
            const WffPlan &P = *plans[i0 + k];
            if (P.fft_L != L || !P.use_colfft() || P.prec != GLSU_F32 || P.pitch % nc != 0)
                return fail(GLSU_ERR_INVALID, "batched column sweep: plans of one FFT length only");
            const double N = 1.0 / P.inv_norm;
            colfft::BatchSeq &q = tab.seq[k];
            q.R = (const float2 *)P.d_R;
            q.C = (float2 *)P.d_C;
            q.khat = (const float2 *)P.d_khat;
            q.thr = (const float *)P.d_thr;
            q.H = P.H;
            q.pitch = P.pitch;
            q.nfy = P.nfy;
            q.ngroups = P.pitch / nc;
            q.LN = (float)(L * N);
            q.out_scale = (float)(1.0 / ((double)L * L * N));
            q.item0 = nitems;
            q.pad_ = 0;
            nitems += q.ngroups * P.nfx;
        }
        const float2 *tw = (const float2 *)plans[i0]->d_tw;
        int rc = colfft::launch_batch_small(L, tab, m, nitems, tw, 0, s);
        if (rc == GLSU_ERR_UNSUPPORTED) rc = colfft::launch_batch_mid(L, tab, m, nitems, tw, 0, s);
        if (rc == GLSU_ERR_UNSUPPORTED) rc = colfft::launch_batch_large(L, tab, m, nitems, tw, 0, s);
        if (rc == GLSU_ERR_UNSUPPORTED) return fail(GLSU_ERR_UNSUPPORTED, "no compiled FFT plan for this length");
        GLSU_TRY(rc);
    }
    return GLSU_OK;
}

// ---------------------------------------------------------------------------
// autotuner
// ---------------------------------------------------------------------------
// GLSU_METHOD_AUTO (the default) decides from the shape alone, with a cost
// model of the two column sweeps (model_ms below), so that the same inputs
// give the same bits in every process and on every box.  The timed search
// below runs only on request (GLSU_METHOD_TIMED, or GLSU_AUTOTUNE=time in
// the environment).
//
// Timed search.  Candidates: the direct column kernel, and the FFT sweep at
// the two shortest compiled transform lengths, then, at the faster length,
// with the other compiled CTA width.  Each is launched once (warm-up), then
// twice between CUDA events on the plan's own buffers; the kernels have no
// data-dependent control flow, so the buffers' contents do not matter.  The
// FFT is taken only when at least 10% faster than the direct kernel, so
// that near ties keep the direct kernel.  Results are kept per shape for the
// process, so every handle of a shape runs the same kernels.
namespace {
struct TuneKey {
    int v[9];
    bool operator<(const TuneKey &o) const { return std::lexicographical_compare(v, v + 9, o.v, o.v + 9); }
};
struct TuneResult {
    int method, L, nc, order;
    float ms_direct, ms_fft;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneResult> g_tune;

// Throughputs of the column-sweep cost model (WffPlan::model_ms), measured
// on GB300 at 2070 MHz from 256^2 to 2048^2: direct kernel in tap-units per
// second per instantiated half-size; FFT sweep in (length x passes) units
// per second, with the load, window products and store of a column worth
// kModelFftColumnUnits passes; both plus a launch and tail constant.
constexpr double kModelDirectRate30 = 1.1e13;
constexpr double kModelDirectRate45 = 5.5e12;
constexpr double kModelDirectRate60 = 3.95e12;
constexpr double kModelFftRate = 1.35e12;
constexpr double kModelFftColumnUnits = 30.0;
constexpr double kModelLaunchMs = 0.05;
}  // namespace

// Modelled device time (ms) of one full-frame column sweep of this plan.
// Direct kernel: per output pixel, x-frequency and y-frequency, two column
// filters of 2S+1 taps (S the instantiated half-size), the first one also
// over the 2S-row halo of each 128-row tile, at a rate per instantiation.
// FFT sweep: per column and x-frequency, 2 nfy + 2 transforms of length L
// in a number of radix passes.
double WffPlan::model_ms(int m) const
{
    if (m == GLSU_METHOD_FFT) {
        if (fft_L == 0) return 1e30;
        const double units = (double)pitch * nfx * fft_L * (fft_nst * (2.0 * nfy + 2.0) + kModelFftColumnUnits);
        return units / kModelFftRate * 1e3 + kModelLaunchMs;
    }
    const int S = syi;
    const double taps = (2.0 * S + 1.0) * (2.0 + 2.0 * S / 128.0);
    const double rate = S <= 30 ? kModelDirectRate30 : (S <= 45 ? kModelDirectRate45 : kModelDirectRate60);
    return (double)pitch * H * nfx * nfy * taps / rate * 1e3 + kModelLaunchMs;
}

// AUTO without timing: the shortest compiled transform length (built by
// init_colfft), its default CTA width, and the FFT sweep when its modelled
// time is below 0.9 x the direct kernel's.
int WffPlan::choose_by_model()
{
    auto_method = GLSU_METHOD_DIRECT;
    if (prec != GLSU_F32 || fft_L == 0 || d_khat == nullptr) return GLSU_OK;
    int L;
    if (length_candidates(H + 2 * sy, &L, 1) == 1 && L != fft_L) GLSU_TRY(build_colfft(L));
    colfft::LenInfo li;
    colfft::len_info(fft_L, &li);
    GLSU_TRY(set_fft_plan(li.ncol_default, 0));
    tune_ms_direct = (float)model_ms(GLSU_METHOD_DIRECT);
    tune_ms_fft = (float)model_ms(GLSU_METHOD_FFT);
    if (tune_ms_fft < 0.9f * tune_ms_direct) auto_method = GLSU_METHOD_FFT;
    return GLSU_OK;
}

int WffPlan::autotune(cudaStream_t s)
{
    tuned = true;
    timed = false;
    auto_method = GLSU_METHOD_DIRECT;
    tune_ms_direct = tune_ms_fft = 0;
    if (prec != GLSU_F32 || fft_L == 0 || d_khat == nullptr) return GLSU_OK;
    const char *env = std::getenv("GLSU_AUTOTUNE");
    if (env && env[0] == '0') return GLSU_OK;
    const bool want_timing = method == GLSU_METHOD_TIMED || (env && std::strcmp(env, "time") == 0);
    if (!want_timing) return choose_by_model();
    timed = true;
    const TuneKey key{{W, H, pitch, sx, sy, nfx, nfy, H + 2 * sy, (int)(1000 * p.wyl + 0.5)}};
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(key);
    if (it == g_tune.end()) {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
            if (e0) cudaEventDestroy(e0);
            return fail(GLSU_ERR_CUDA, "cudaEventCreate failed");
        }
        const int saved = method;
        int rc = GLSU_OK;
        auto time_it = [&](int m, float *ms) {
            method = m;
            for (int k = 0; k < 3 && rc == GLSU_OK; k++) {
                if (k == 1 && cudaEventRecord(e0, s) != cudaSuccess) rc = fail(GLSU_ERR_CUDA, "cudaEventRecord");
                if (rc == GLSU_OK) rc = launch_column_sweep(*this, s);
            }
            if (rc == GLSU_OK && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                                  cudaEventElapsedTime(ms, e0, e1) != cudaSuccess))
                rc = fail(GLSU_ERR_CUDA, "timing a column-sweep candidate failed");
            *ms *= 0.5f;
        };
        TuneResult r{GLSU_METHOD_DIRECT, fft_L, fft_nc, fft_order, 0.f, 0.f};
        time_it(GLSU_METHOD_DIRECT, &r.ms_direct);
        float best = -1.f;
        int lens[2];
        const int nl = length_candidates(H + 2 * sy, lens, 2);
        for (int j = 0; j < nl && rc == GLSU_OK; j++) {
            if (build_colfft(lens[j]) != GLSU_OK) continue;
            float ms = 0;
            time_it(GLSU_METHOD_FFT, &ms);
            if (rc == GLSU_OK && (best < 0 || ms < best)) {
                best = ms;
                r.L = lens[j];
                r.nc = fft_nc;
                r.order = fft_order;
            }
        }
        if (rc == GLSU_OK && r.L != fft_L) rc = build_colfft(r.L);
        if (rc == GLSU_OK && best > 0 && set_fft_plan(2 * fft_nc, 0) == GLSU_OK) {
            float ms = 0;
            time_it(GLSU_METHOD_FFT, &ms);
            if (rc == GLSU_OK && ms < best) {
                best = ms;
                r.nc = fft_nc;
            }
        }
        set_error(std::string());  // variants that did not fit leave no message
        method = saved;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc != GLSU_OK) return rc;
        r.ms_fft = best;
        if (best > 0 && best < 0.9f * r.ms_direct) r.method = GLSU_METHOD_FFT;
        it = g_tune.emplace(key, r).first;
    }
    const TuneResult &r = it->second;
    auto_method = r.method;
    tune_ms_direct = r.ms_direct;
    tune_ms_fft = r.ms_fft;
    if (r.L != fft_L) GLSU_TRY(build_colfft(r.L));
    return set_fft_plan(r.nc, r.order);
}

}  // namespace glsu
