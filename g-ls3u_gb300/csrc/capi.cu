// capi.cu -- the C ABI (include/glsu.h): handles, buffers, streams, timing.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "func_attr.hpp"
#include "glsu_internal.cuh"
#include "sur_net.cuh"

namespace glsu {

static thread_local std::string g_err;

void set_error(const std::string &msg) { g_err = msg; }

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return GLSU_ERR_ALLOC;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return GLSU_ERR_NO_DEVICE;
    return GLSU_ERR_CUDA;
}

static FuncAttrCache g_attr;

int raise_smem_limit(const void *func, int bytes, int carveout)
{
    int dev = 0;
    GLSU_CUDA_TRY(cudaGetDevice(&dev));
    if (!g_attr.needs(func, dev, bytes)) return GLSU_OK;
    // a refused attribute would stay the runtime's last error and surface at
    // the next launch check: clear it and report it here
    if (cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(GLSU_ERR_UNSUPPORTED,
                    "a kernel's dynamic shared memory (" + std::to_string(bytes) + " bytes) exceeds the device limit");
    }
    if (carveout >= 0 &&
        cudaFuncSetAttribute(func, cudaFuncAttributePreferredSharedMemoryCarveout, carveout) != cudaSuccess) {
        cudaGetLastError();
        return fail(GLSU_ERR_CUDA, "cudaFuncSetAttribute (shared-memory carveout) failed");
    }
    g_attr.done(func, dev, bytes);
    return GLSU_OK;
}

int device_smem_optin()
{
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int device_sm_count()
{
    static std::mutex mu;
    static std::map<int, int> counts;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    std::lock_guard<std::mutex> lock(mu);
    auto it = counts.find(dev);
    if (it != counts.end()) return it->second;
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) {
        cudaGetLastError();
        n = 1;
    }
    counts[dev] = n;
    return n;
}

int wff_count_public(double lo, double hi, double step, int prec);

// Is p a page-locked (pinned or registered) host pointer?
static bool is_pinned(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

static size_t elem_size(int t)
{
    return t == GLSU_U8 ? 1 : (t == GLSU_F32 ? 4 : (t == GLSU_F64 ? 8 : 0));
}

}  // namespace glsu

using namespace glsu;

// ===========================================================================
// handles
// ===========================================================================
struct glsu_wff {
    WffPlan plan;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

struct glsu_wfr {
    WffPlan plan;
    WfrBuffers buf;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

struct glsu_dpra {
    int prec = GLSU_F32;
    int W = 0, H = 0, rr = 1, r = 1;
    WffPlan wff;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    void *d_img = nullptr;  // one frame, 8 bytes per pixel
    void *d_z = nullptr;    // exp(j dphi), complex
    void *d_phi[4] = {nullptr, nullptr, nullptr, nullptr};  // ref, curr, dphi_ref, dphi
    void *h_in = nullptr, *h_out = nullptr;                 // pinned staging
    bool synced = true;  // phi_curr/dphi equal phi_ref/dphi_ref (after an update)
    bool timing = false;
    bool unwrap = false;  // MATLAB fp_ls3u semantics: dphi = dphi_ref + unwrap(t)
    int unwrap_row = -1, unwrap_col = -1;
    int ls_method = GLSU_LS_FLOAT_FLOAT;
    int ls_tile = 0;  // output tile of the float-float LS: 0 = 32 x 16, 1 = 32 x 8, 2 = 32 x 32
    cudaEvent_t ev[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    int frames_done = 0;
    // pipelined sequence over pinned host buffers: frame slot s uses
    // d_seq_img[s] (slot 0 is d_img) and output ring d_ring[s]
    cudaStream_t s_in = nullptr, s_out = nullptr;
    void *d_seq_img1 = nullptr, *d_ring[2] = {nullptr, nullptr};
    cudaEvent_t ev_in[2] = {nullptr, nullptr}, ev_comp[2] = {nullptr, nullptr}, ev_out[2] = {nullptr, nullptr};
    // surrogate form: network output, probes, per-tile fallback.  The
    // probes' exact WFF2 sweep runs on s_probe concurrently with the network
    // (fork after the LS stage, join before the residuals); ev_p time it.
    SurNet *sur = nullptr;
    cudaStream_t s_probe = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_p[2] = {nullptr, nullptr};
    bool probe_overlap = true;
    int overlap_conv_ctas = 0;  // cap of tensor-core CTAs per SM while the probe sweep runs beside them (0: none)
    // CUDA-graph replay of the per-frame work (opt-in): one executable graph
    // per (input buffer, image type, parity of the exchanged phase buffers)
    struct FrameGraph {
        const void *in = nullptr;
        int type = -1, parity = -1;
        cudaGraphExec_t exec = nullptr;
    };
    bool use_graph = false;
    int phi_parity = 0;  // flips with every exchange of the reference / current buffers
    FrameGraph graphs[4];
    int graph_next = 0;
    bool graph_warm = false;  // one eager frame ran since the graphs were last dropped
    int batch_index = 0;      // frames run through glsu_dpra_batch_step
    void *d_filt = nullptr;  // complex H*W: the filtered field (surrogate, then fallback tiles)
    int sur_tile = 0, sur_patch = 0, sur_ntx = 0, sur_nty = 0;
    double sur_tol = 0;
    ProbeOut probe;
};

static void dpra_surrogate_release(glsu_dpra *h);

struct glsu_aia {
    int M = 0, cols = 0, rows = 0, N = 0;
    AiaDev dev;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    void *d_frames = nullptr;  // M*N*4 bytes
    float *d_phi = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
};

// ===========================================================================
// utilities
// ===========================================================================
extern "C" const char *glsu_last_error(void) { return g_err.c_str(); }

extern "C" int glsu_version(void) { return 100; }

extern "C" int glsu_opt_fft_size(int x)
{
    // even sizes 2^a 3^b 5^c 7^d up to 4096 (WFT/WFT.h:18-32), first >= x
    if (x > 4096) return -1;
    for (int v = (x < 2 ? 2 : x + (x & 1)); v <= 4096; v += 2) {
        int t = v;
        while (t % 2 == 0) t /= 2;
        while (t % 3 == 0) t /= 3;
        while (t % 5 == 0) t /= 5;
        while (t % 7 == 0) t /= 7;
        if (t == 1) return v;
    }
    return -1;
}

extern "C" int glsu_wft_default_params(int wft_type, glsu_wff_params *p)
{
    if (!p) return fail(GLSU_ERR_INVALID, "null params");
    if (wft_type == GLSU_WFT_WFF) {
        // WFT/WFT2_CUDAf.cu:852-861 (float arithmetic as in WFT2_CUDAF)
        const float s = 10.0f;
        p->sigma_x = s; p->wxl = -2.0f - 3.0f / s; p->wxi = 1.0f / s; p->wxh = 2.0f + 3.0f / s;
        p->sigma_y = s; p->wyl = -2.0f - 3.0f / s; p->wyi = 1.0f / s; p->wyh = 2.0f + 3.0f / s;
        p->thr = -1;
        return GLSU_OK;
    }
    if (wft_type == GLSU_WFT_WFR) {
        p->sigma_x = 10; p->wxl = -2; p->wxi = 0.025f; p->wxh = 2;
        p->sigma_y = 10; p->wyl = -2; p->wyi = 0.025f; p->wyh = 2;
        p->thr = -1;
        return GLSU_OK;
    }
    return fail(GLSU_ERR_INVALID, "unknown WFT type");
}

extern "C" int glsu_dpra_default_wff_params(glsu_wff_params *p)
{
    if (!p) return fail(GLSU_ERR_INVALID, "null params");
    // DPRA/dpra_cudaf.cu:116-118 (float literals)
    p->sigma_x = 20; p->wxl = -0.15f; p->wxh = 0.15f; p->wxi = 0.05f;
    p->sigma_y = 20; p->wyl = -0.15f; p->wyh = 0.15f; p->wyi = 0.05f;
    p->thr = 15;
    return GLSU_OK;
}

extern "C" int glsu_wff_count(double lo, double hi, double step, int precision)
{
    if (!(step > 0)) return fail(GLSU_ERR_INVALID, "step must be positive");
    return wff_count_public(lo, hi, step, precision);
}

// splitmix64 + Box-Muller: deterministic N(0,1) draws for the AIA start
static uint64_t splitmix64(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

extern "C" int glsu_aia_random_deltas(int M, uint64_t seed, float *deltas)
{
    if (M < 1 || !deltas) return fail(GLSU_ERR_INVALID, "bad arguments");
    uint64_t s = seed;
    deltas[0] = 0;
    for (int i = 1; i < M; i++) {
        const double u1 = ((splitmix64(s) >> 11) + 1) * (1.0 / 9007199254740993.0);
        const double u2 = (splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
        deltas[i] = (float)(std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2));
    }
    return GLSU_OK;
}

// ===========================================================================
// WFF2
// ===========================================================================
static int wff_setup_stream(cudaStream_t *s, bool *own)
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(GLSU_ERR_NO_DEVICE, "no CUDA device visible");
    }
    GLSU_CUDA_TRY(cudaStreamCreateWithFlags(s, cudaStreamNonBlocking));
    *own = true;
    return GLSU_OK;
}

extern "C" int glsu_wff_create(glsu_wff **out, int precision, int width, int height, const glsu_wff_params *p)
{
    if (!out) return fail(GLSU_ERR_INVALID, "null handle pointer");
    *out = nullptr;
    glsu_wff_params prm;
    if (p) prm = *p;
    else glsu_wft_default_params(GLSU_WFT_WFF, &prm);
    glsu_wff *h = new glsu_wff();
    int rc = h->plan.init(precision, width, height, prm);
    if (rc == GLSU_OK) rc = wff_setup_stream(&h->stream, &h->own_stream);
    if (rc == GLSU_OK) rc = h->plan.alloc_device();
    if (rc == GLSU_OK) rc = h->plan.upload_tables(h->stream);
    if (rc == GLSU_OK) rc = h->plan.make_tensor_map();
    if (rc == GLSU_OK) rc = h->plan.init_colfft();
    if (rc == GLSU_OK) rc = h->plan.autotune(h->stream);
    if (rc == GLSU_OK && (cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess))
        rc = fail(GLSU_ERR_CUDA, "cudaEventCreate failed");
    if (rc != GLSU_OK) {
        glsu_wff_destroy(h);
        return rc;
    }
    *out = h;
    return GLSU_OK;
}

extern "C" int glsu_wff_destroy(glsu_wff *h)
{
    if (!h) return GLSU_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    h->plan.release();
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return GLSU_OK;
}

extern "C" int glsu_wff_set_stream(glsu_wff *h, void *stream)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    if (h->own_stream && h->stream) {
        cudaStreamSynchronize(h->stream);
        cudaStreamDestroy(h->stream);
    }
    h->stream = (cudaStream_t)stream;
    h->own_stream = false;
    return GLSU_OK;
}

extern "C" int glsu_wff_run_async(glsu_wff *h, const void *d_f, void *d_filtered)
{
    if (!h || !d_f || !d_filtered) return fail(GLSU_ERR_INVALID, "null argument");
    return h->plan.enqueue(h->stream, d_f, d_filtered, 0, nullptr, nullptr, nullptr, nullptr, nullptr);
}

// ===========================================================================
// WFR2
// ===========================================================================
extern "C" int glsu_wfr_create(glsu_wfr **out, int precision, int width, int height, const glsu_wff_params *p)
{
    if (!out) return fail(GLSU_ERR_INVALID, "null handle pointer");
    *out = nullptr;
    glsu_wff_params prm;
    if (p) prm = *p;
    else glsu_wft_default_params(GLSU_WFT_WFR, &prm);
    prm.thr = 0;  // not used by WFR2
    glsu_wfr *h = new glsu_wfr();
    int rc = h->plan.init(precision, width, height, prm);
    if (rc == GLSU_OK) rc = wff_setup_stream(&h->stream, &h->own_stream);
    if (rc == GLSU_OK) rc = h->plan.alloc_device();
    if (rc == GLSU_OK) rc = h->plan.upload_tables(h->stream);
    if (rc == GLSU_OK) rc = h->plan.make_tensor_map();
    if (rc == GLSU_OK) rc = h->buf.alloc(h->plan);
    if (rc == GLSU_OK && (cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess))
        rc = fail(GLSU_ERR_CUDA, "cudaEventCreate failed");
    if (rc != GLSU_OK) {
        glsu_wfr_destroy(h);
        return rc;
    }
    *out = h;
    return GLSU_OK;
}

extern "C" int glsu_wfr_destroy(glsu_wfr *h)
{
    if (!h) return GLSU_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    h->buf.release();
    h->plan.release();
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return GLSU_OK;
}

extern "C" int glsu_wfr_set_stream(glsu_wfr *h, void *stream)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    if (h->own_stream && h->stream) {
        cudaStreamSynchronize(h->stream);
        cudaStreamDestroy(h->stream);
    }
    h->stream = (cudaStream_t)stream;
    h->own_stream = false;
    return GLSU_OK;
}

static int wfr_check_results(const glsu_wfr_results *z)
{
    if (!z || !z->wx || !z->wy || !z->phase || !z->phase_comp || !z->b || !z->r || !z->cxx || !z->cyy)
        return fail(GLSU_ERR_INVALID, "null WFR result map");
    return GLSU_OK;
}

extern "C" int glsu_wfr_run_async(glsu_wfr *h, const void *d_f, const glsu_wfr_results *z)
{
    if (!h || !d_f) return fail(GLSU_ERR_INVALID, "null argument");
    GLSU_TRY(wfr_check_results(z));
    return enqueue_wfr(h->plan, h->buf, h->stream, d_f, *z);
}

extern "C" int glsu_wfr_run(glsu_wfr *h, const void *d_f, const glsu_wfr_results *z, double *time_ms)
{
    if (!h || !d_f) return fail(GLSU_ERR_INVALID, "null argument");
    GLSU_TRY(wfr_check_results(z));
    GLSU_CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
    GLSU_TRY(enqueue_wfr(h->plan, h->buf, h->stream, d_f, *z));
    GLSU_CUDA_TRY(cudaEventRecord(h->ev1, h->stream));
    GLSU_CUDA_TRY(cudaEventSynchronize(h->ev1));
    GLSU_TRY(h->plan.check_device_error(h->stream));
    if (time_ms) {
        float ms = 0;
        GLSU_CUDA_TRY(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
        *time_ms = ms;
    }
    return GLSU_OK;
}

extern "C" int glsu_wff_run(glsu_wff *h, const void *d_f, void *d_filtered, double *time_ms)
{
    if (!h || !d_f || !d_filtered) return fail(GLSU_ERR_INVALID, "null argument");
    GLSU_CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
    GLSU_TRY(h->plan.enqueue(h->stream, d_f, d_filtered, 0, nullptr, nullptr, nullptr, nullptr, nullptr));
    GLSU_CUDA_TRY(cudaEventRecord(h->ev1, h->stream));
    GLSU_TRY(h->plan.check_device_error(h->stream));
    if (time_ms) {
        float ms = 0;
        GLSU_CUDA_TRY(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
        *time_ms = ms;
    }
    return GLSU_OK;
}

extern "C" int glsu_wff_threshold(glsu_wff *h, double *thr)
{
    if (!h || !thr) return fail(GLSU_ERR_INVALID, "null argument");
    if (h->plan.p.thr >= 0) {
        *thr = h->plan.p.thr;
        return GLSU_OK;
    }
    if (!h->plan.thr_ready) {
        *thr = -1;
        return GLSU_OK;
    }
    GLSU_CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (h->plan.prec == GLSU_F32) {
        float t;
        GLSU_CUDA_TRY(cudaMemcpy(&t, h->plan.d_thr, sizeof(float), cudaMemcpyDeviceToHost));
        *thr = t;
    } else {
        GLSU_CUDA_TRY(cudaMemcpy(thr, h->plan.d_thr, sizeof(double), cudaMemcpyDeviceToHost));
    }
    return GLSU_OK;
}

static int set_method(WffPlan &P, int method, cudaStream_t s)
{
    if (method != GLSU_METHOD_AUTO && method != GLSU_METHOD_DIRECT && method != GLSU_METHOD_FFT &&
        method != GLSU_METHOD_TIMED)
        return fail(GLSU_ERR_INVALID, "unknown column-sweep method");
    if (method == GLSU_METHOD_FFT && P.fft_L == 0)
        return fail(GLSU_ERR_UNSUPPORTED, "no shared-memory FFT plan for this handle (FP64, or no transform length)");
    GLSU_CUDA_TRY(cudaStreamSynchronize(s));
    P.method = method;
    if (method == GLSU_METHOD_AUTO || method == GLSU_METHOD_TIMED) return P.autotune(s);
    return GLSU_OK;
}

static void get_tuning(const WffPlan &P, glsu_wff_tuning *t)
{
    t->method = P.column_method() == GLSU_METHOD_FFT && P.fft_L > 0 ? GLSU_METHOD_FFT : GLSU_METHOD_DIRECT;
    t->fft_length = P.fft_L;
    t->fft_columns = P.fft_nc;
    t->fft_radix_order = P.fft_order;
    t->tuned = P.tuned ? (P.timed ? 1 : 2) : 0;
    t->ms_direct = P.tune_ms_direct;
    t->ms_fft = P.tune_ms_fft;
}

extern "C" int glsu_wff_set_method(glsu_wff *h, int method)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    return set_method(h->plan, method, h->stream);
}

extern "C" int glsu_wff_get_tuning(const glsu_wff *h, glsu_wff_tuning *t)
{
    if (!h || !t) return fail(GLSU_ERR_INVALID, "null argument");
    get_tuning(h->plan, t);
    return GLSU_OK;
}

extern "C" int glsu_wff_set_fft_plan(glsu_wff *h, int columns_per_cta, int radix_order)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    GLSU_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return h->plan.set_fft_plan(columns_per_cta, radix_order);
}

extern "C" int glsu_wff_set_fft_length(glsu_wff *h, int length)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    if (h->plan.fft_L == 0) return fail(GLSU_ERR_UNSUPPORTED, "no shared-memory FFT plan for this handle");
    GLSU_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return h->plan.build_colfft(length);
}

extern "C" int glsu_wff_fft_lengths(const glsu_wff *h, int *lengths, int n)
{
    if (!h || (!lengths && n > 0) || n < 0) return fail(GLSU_ERR_INVALID, "bad argument");
    return fft_length_candidates(h->plan, lengths, n);
}

// Executable frame graphs capture the handle's configuration and buffers:
// every change of either drops them.
static void dpra_drop_graphs(glsu_dpra *h)
{
    bool any = false;
    for (auto &g : h->graphs) any = any || g.exec;
    if (any && h->stream) cudaStreamSynchronize(h->stream);  // no replay of them still in flight
    for (auto &g : h->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = glsu_dpra::FrameGraph();
    }
    h->graph_next = 0;
    h->graph_warm = false;
}

extern "C" int glsu_dpra_set_method(glsu_dpra *h, int method)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    dpra_drop_graphs(h);
    return set_method(h->wff, method, h->stream);
}

extern "C" int glsu_dpra_get_tuning(const glsu_dpra *h, glsu_wff_tuning *t)
{
    if (!h || !t) return fail(GLSU_ERR_INVALID, "null argument");
    get_tuning(h->wff, t);
    return GLSU_OK;
}

extern "C" int glsu_wff_padded_size(const glsu_wff *h, int *pw, int *ph)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    if (pw) *pw = h->plan.Wp;
    if (ph) *ph = h->plan.Hp;
    return GLSU_OK;
}

// ===========================================================================
// DPRA
// ===========================================================================
extern "C" int glsu_dpra_create(glsu_dpra **out, int precision, const void *h_phi0, int width, int height,
                                int ref_update_rate, int window_radius, const glsu_wff_params *wff)
{
    if (!out) return fail(GLSU_ERR_INVALID, "null handle pointer");
    *out = nullptr;
    if (!h_phi0) return fail(GLSU_ERR_INVALID, "null initial phase");
    if (ref_update_rate < 1) return fail(GLSU_ERR_INVALID, "reference update rate must be >= 1");
    if (window_radius < 1 || window_radius > 8) return fail(GLSU_ERR_UNSUPPORTED, "DPRA window radius must be 1..8");
    glsu_wff_params prm;
    if (wff) prm = *wff;
    else glsu_dpra_default_wff_params(&prm);
    glsu_dpra *h = new glsu_dpra();
    h->prec = precision;
    h->W = width;
    h->H = height;
    h->rr = ref_update_rate;
    h->r = window_radius;
    int rc = h->wff.init(precision, width, height, prm);
    if (rc == GLSU_OK) rc = wff_setup_stream(&h->stream, &h->own_stream);
    if (rc == GLSU_OK) rc = h->wff.alloc_device();
    if (rc == GLSU_OK) rc = h->wff.upload_tables(h->stream);
    if (rc == GLSU_OK) rc = h->wff.make_tensor_map();
    if (rc == GLSU_OK) rc = h->wff.init_colfft();
    if (rc == GLSU_OK) rc = h->wff.autotune(h->stream);
    const size_t N = (size_t)width * height;
    const size_t es = precision == GLSU_F32 ? 4 : 8;
    if (rc == GLSU_OK) {
        bool ok = cudaMalloc(&h->d_img, 8 * N) == cudaSuccess && cudaMalloc(&h->d_z, 2 * es * N) == cudaSuccess;
        for (int k = 0; k < 4 && ok; k++) ok = cudaMalloc(&h->d_phi[k], es * N) == cudaSuccess;
        ok = ok && cudaMallocHost(&h->h_in, 8 * N) == cudaSuccess && cudaMallocHost(&h->h_out, es * N) == cudaSuccess;
        if (!ok) rc = fail(GLSU_ERR_ALLOC, "DPRA buffer allocation failed");
    }
    if (rc == GLSU_OK) {
        if (cudaMemcpy(h->d_phi[GLSU_PHI_REF], h_phi0, es * N, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(h->d_phi[GLSU_PHI_CURR], h_phi0, es * N, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemset(h->d_phi[GLSU_DPHI_REF], 0, es * N) != cudaSuccess ||
            cudaMemset(h->d_phi[GLSU_DPHI], 0, es * N) != cudaSuccess)
            rc = fail(GLSU_ERR_CUDA, "initial phase upload failed");
    }
    for (int k = 0; k < 8 && rc == GLSU_OK; k++)
        if (cudaEventCreate(&h->ev[k]) != cudaSuccess) rc = fail(GLSU_ERR_CUDA, "cudaEventCreate failed");
    if (rc == GLSU_OK && (cudaEventCreate(&h->t0) != cudaSuccess || cudaEventCreate(&h->t1) != cudaSuccess))
        rc = fail(GLSU_ERR_CUDA, "cudaEventCreate failed");
    if (rc != GLSU_OK) {
        glsu_dpra_destroy(h);
        return rc;
    }
    *out = h;
    return GLSU_OK;
}

extern "C" int glsu_dpra_destroy(glsu_dpra *h)
{
    if (!h) return GLSU_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    dpra_drop_graphs(h);
    h->wff.release();
    cudaFree(h->d_img);
    cudaFree(h->d_z);
    for (int k = 0; k < 4; k++) cudaFree(h->d_phi[k]);
    cudaFreeHost(h->h_in);
    cudaFreeHost(h->h_out);
    for (int k = 0; k < 8; k++)
        if (h->ev[k]) cudaEventDestroy(h->ev[k]);
    if (h->t0) cudaEventDestroy(h->t0);
    if (h->t1) cudaEventDestroy(h->t1);
    if (h->s_in) cudaStreamSynchronize(h->s_in);
    if (h->s_out) cudaStreamSynchronize(h->s_out);
    cudaFree(h->d_seq_img1);
    for (int s = 0; s < 2; s++) {
        cudaFree(h->d_ring[s]);
        if (h->ev_in[s]) cudaEventDestroy(h->ev_in[s]);
        if (h->ev_comp[s]) cudaEventDestroy(h->ev_comp[s]);
        if (h->ev_out[s]) cudaEventDestroy(h->ev_out[s]);
    }
    if (h->s_in) cudaStreamDestroy(h->s_in);
    if (h->s_out) cudaStreamDestroy(h->s_out);
    dpra_surrogate_release(h);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return GLSU_OK;
}

extern "C" int glsu_dpra_set_stream(glsu_dpra *h, void *stream)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    dpra_drop_graphs(h);
    if (h->own_stream && h->stream) {
        cudaStreamSynchronize(h->stream);
        cudaStreamDestroy(h->stream);
    }
    h->stream = (cudaStream_t)stream;
    h->own_stream = false;
    return GLSU_OK;
}

static int dpra_check_type(glsu_dpra *h, int img_type)
{
    if (img_type == GLSU_U8 || img_type == GLSU_F32) return GLSU_OK;
    if (img_type == GLSU_F64 && h->prec == GLSU_F64) return GLSU_OK;
    return fail(GLSU_ERR_INVALID, "frame type must be GLSU_U8, GLSU_F32 or (FP64 handles) GLSU_F64");
}

static void dpra_surrogate_release(glsu_dpra *h)
{
    if (h->sur) {
        h->sur->release();
        delete h->sur;
        h->sur = nullptr;
    }
    if (h->s_probe) {
        cudaStreamSynchronize(h->s_probe);
        cudaStreamDestroy(h->s_probe);
        h->s_probe = nullptr;
    }
    cudaEvent_t *evs[] = {&h->ev_fork, &h->ev_join, &h->ev_p[0], &h->ev_p[1]};
    for (cudaEvent_t *e : evs)
        if (*e) {
            cudaEventDestroy(*e);
            *e = nullptr;
        }
    cudaFree(h->d_filt);
    cudaFree(h->probe.partial);
    cudaFree(h->probe.sites);
    cudaFree(h->probe.resid);
    cudaFree(h->probe.flags);
    cudaFree(h->probe.counts);
    cudaFree(h->probe.rows);
    cudaFree(h->probe.seed);
    h->d_filt = nullptr;
    h->probe = ProbeOut();
}

// Surrogate form of one frame after the LS stage (d_z): the exact WFF2 probe
// sweep forks onto s_probe and runs beside the network; the residuals join
// behind it, then plain WFF2 on flagged tiles and the phase update.  Stage
// events: ev[0] before the network, ev[6] after its layer 0, ev[7] after its
// six tensor-core layers, ev[1] after the network, ev[2] after the join and
// the residuals, ev[3] after fallback and update; ev_p around the sweep.
static int dpra_surrogate_frame(glsu_dpra *h, cudaEvent_t *ev)
{
    const bool probe = h->sur_tol > 0;
    const bool overlap = probe && h->probe_overlap;
    if (overlap) {
        GLSU_CUDA_TRY(cudaEventRecord(h->ev_fork, h->stream));
        GLSU_CUDA_TRY(cudaStreamWaitEvent(h->s_probe, h->ev_fork, 0));
        if (ev) GLSU_CUDA_TRY(cudaEventRecord(h->ev_p[0], h->s_probe));
        GLSU_TRY(h->wff.enqueue_probe_sweep(h->s_probe, h->d_z, h->sur_tile, h->sur_patch, (uint32_t)h->frames_done,
                                            h->probe));
        if (ev) GLSU_CUDA_TRY(cudaEventRecord(h->ev_p[1], h->s_probe));
        GLSU_CUDA_TRY(cudaEventRecord(h->ev_join, h->s_probe));
    }
    if (ev) GLSU_CUDA_TRY(cudaEventRecord(ev[0], h->stream));
    h->sur->stream = h->stream;
    h->sur->conv_ctas_per_sm = overlap ? h->overlap_conv_ctas : 0;
    GLSU_TRY(h->sur->forward(h->d_z, h->d_filt, ev ? ev + 6 : nullptr));
    if (ev) GLSU_CUDA_TRY(cudaEventRecord(ev[1], h->stream));
    if (probe) {
        if (overlap) {
            GLSU_CUDA_TRY(cudaStreamWaitEvent(h->stream, h->ev_join, 0));
        } else {
            if (ev) GLSU_CUDA_TRY(cudaEventRecord(h->ev_p[0], h->stream));
            GLSU_TRY(h->wff.enqueue_probe_sweep(h->stream, h->d_z, h->sur_tile, h->sur_patch,
                                                (uint32_t)h->frames_done, h->probe));
            if (ev) GLSU_CUDA_TRY(cudaEventRecord(h->ev_p[1], h->stream));
        }
        GLSU_TRY(h->wff.enqueue_probe_resid(h->stream, h->d_filt, h->sur_tol, h->probe));
        if (ev) GLSU_CUDA_TRY(cudaEventRecord(ev[2], h->stream));
        TileMask m;
        m.flags = h->probe.flags;
        m.tile = h->sur_tile;
        m.ntx = h->sur_ntx;
        m.nty = h->sur_nty;
        h->wff.mask = m;
        const int rc = h->wff.enqueue(h->stream, h->d_z, h->d_filt, 0, nullptr, nullptr, nullptr, nullptr, nullptr);
        h->wff.mask = TileMask();
        GLSU_TRY(rc);
    } else if (ev) {
        GLSU_CUDA_TRY(cudaEventRecord(ev[2], h->stream));
    }
    GLSU_TRY(launch_dpra_update(h->prec, h->d_filt, h->d_phi[GLSU_PHI_REF], h->unwrap ? nullptr : h->d_phi[GLSU_DPHI_REF],
                                h->d_phi[GLSU_PHI_CURR], h->d_phi[GLSU_DPHI], h->W * h->H, h->stream));
    if (ev) GLSU_CUDA_TRY(cudaEventRecord(ev[3], h->stream));
    return GLSU_OK;
}

extern "C" int glsu_dpra_set_probe_overlap(glsu_dpra *h, int enable, int conv_ctas_per_sm)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    dpra_drop_graphs(h);
    if (conv_ctas_per_sm < 0) return fail(GLSU_ERR_INVALID, "negative CTA cap");
    GLSU_CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->probe_overlap = enable != 0;
    h->overlap_conv_ctas = conv_ctas_per_sm;
    return GLSU_OK;
}

extern "C" int glsu_dpra_set_surrogate(glsu_dpra *h, const float *h_params, const int *dilations, int tile,
                                       int patch, double tol)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    dpra_drop_graphs(h);
    GLSU_CUDA_TRY(cudaStreamSynchronize(h->stream));
    dpra_surrogate_release(h);
    if (!h_params) return GLSU_OK;
    if (h->prec != GLSU_F32) return fail(GLSU_ERR_UNSUPPORTED, "the surrogate form is FP32");
    const int s_inst = std::max(h->wff.sxi, h->wff.syi);
    if (tol > 0 && s_inst > 45)
        return fail(GLSU_ERR_UNSUPPORTED, "the WFF2 probe supports window half-sizes up to 45");
    if (tol > 0 && patch == 0) patch = probe_patch_for_half(s_inst);
    if (tol > 0 && (tile < 1 || patch != probe_patch_for_half(s_inst) || patch > tile))
        return fail(GLSU_ERR_INVALID, "probe patch must be 0 (default) or the window's patch size, within the tile");
    const size_t N = (size_t)h->W * h->H;
    h->sur = new SurNet();
    h->sur->stream = h->stream;
    int rc = h->sur->init(1, h->W, h->H, dilations, false);
    if (rc == GLSU_OK) rc = h->sur->set_params(h_params);
    if (rc == GLSU_OK && cudaMalloc(&h->d_filt, 8 * N) != cudaSuccess) rc = fail(GLSU_ERR_ALLOC, "allocation failed");
    h->sur_tol = tol;
    if (rc == GLSU_OK && tol > 0) {
        h->sur_tile = tile;
        h->sur_patch = patch;
        h->sur_ntx = (h->W + tile - 1) / tile;
        h->sur_nty = (h->H + tile - 1) / tile;
        const size_t nt = (size_t)h->sur_ntx * h->sur_nty;
        // partials: per tile, wx and part of the wy range (at most 4 parts)
        if (cudaMalloc(&h->probe.partial, nt * h->wff.nfx * 4 * patch * patch * sizeof(float2)) != cudaSuccess ||
            cudaMalloc(&h->probe.sites, nt * sizeof(int2)) != cudaSuccess ||
            cudaMalloc(&h->probe.resid, nt * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&h->probe.flags, nt * sizeof(int)) != cudaSuccess ||
            cudaMalloc(&h->probe.counts, 2 * sizeof(int)) != cudaSuccess ||
            cudaMalloc(&h->probe.rows, nt * h->wff.nfx * probe_rows_elems(s_inst) * sizeof(float2)) != cudaSuccess ||
            cudaMalloc(&h->probe.seed, sizeof(uint32_t)) != cudaSuccess)
            rc = fail(GLSU_ERR_ALLOC, "allocation failed");
        if (rc == GLSU_OK) rc = h->wff.alloc_tile_list();
        if (rc == GLSU_OK && (cudaStreamCreateWithFlags(&h->s_probe, cudaStreamNonBlocking) != cudaSuccess ||
                              cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
                              cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess ||
                              cudaEventCreate(&h->ev_p[0]) != cudaSuccess || cudaEventCreate(&h->ev_p[1]) != cudaSuccess))
            rc = fail(GLSU_ERR_CUDA, "probe stream or event creation failed");
        if (rc == GLSU_OK && (cudaMemset(h->probe.counts, 0, 2 * sizeof(int)) != cudaSuccess ||
                              cudaMemset(h->probe.seed, 0, sizeof(uint32_t)) != cudaSuccess ||
                              cudaMemset(h->probe.resid, 0, nt * sizeof(float)) != cudaSuccess))
            rc = fail(GLSU_ERR_CUDA, "memset failed");
    }
    if (rc != GLSU_OK) dpra_surrogate_release(h);
    return rc;
}

extern "C" int glsu_dpra_surrogate_stats(glsu_dpra *h, long long *tiles_probed, long long *tiles_flagged,
                                         float *h_resid, int *h_sites)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    int c[2] = {0, 0};
    GLSU_CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (h->sur && h->probe.counts) {
        GLSU_CUDA_TRY(cudaMemcpy(c, h->probe.counts, sizeof(c), cudaMemcpyDeviceToHost));
        if (h_resid)
            GLSU_CUDA_TRY(cudaMemcpy(h_resid, h->probe.resid, sizeof(float) * h->sur_ntx * h->sur_nty,
                                     cudaMemcpyDeviceToHost));
        if (h_sites)
            GLSU_CUDA_TRY(cudaMemcpy(h_sites, h->probe.sites, sizeof(int2) * h->sur_ntx * h->sur_nty,
                                     cudaMemcpyDeviceToHost));
    }
    if (tiles_probed) *tiles_probed = c[0];
    if (tiles_flagged) *tiles_flagged = c[1];
    return GLSU_OK;
}

// The device work of one frame on the handle's stream(s): LS, then the plain
// or surrogate form, then the optional unwrapping.
static int dpra_enqueue_frame(glsu_dpra *h, const void *d_img, int img_type)
{
    cudaEvent_t *ev = h->timing ? h->ev : nullptr;
    if (ev) GLSU_CUDA_TRY(cudaEventRecord(ev[4], h->stream));
    GLSU_TRY(launch_dpra_ls(h->prec, img_type, d_img, h->d_phi[GLSU_PHI_REF], h->d_z, h->W, h->H, h->r, h->stream,
                            h->ls_method, h->ls_tile));
    if (h->sur)
        GLSU_TRY(dpra_surrogate_frame(h, ev));
    else
        GLSU_TRY(h->wff.enqueue(h->stream, h->d_z, nullptr, h->unwrap ? 2 : 1, h->d_phi[GLSU_PHI_REF],
                                h->d_phi[GLSU_DPHI_REF], h->d_phi[GLSU_PHI_CURR], h->d_phi[GLSU_DPHI], ev));
    if (h->unwrap)
        GLSU_TRY(launch_unwrap(h->prec, h->d_phi[GLSU_DPHI], h->d_phi[GLSU_DPHI_REF], h->W, h->H, h->unwrap_row,
                               h->unwrap_col, h->stream));
    return GLSU_OK;
}

// Graph mode: the frame's work captured once per (input buffer, type,
// parity) and replayed.  Inputs outside the handle's own frame buffers are
// copied into its first one.
static int dpra_graph_frame(glsu_dpra *h, const void *d_img, int img_type)
{
    const void *in = d_img;
    if (in != h->d_img && in != h->d_seq_img1) {
        GLSU_CUDA_TRY(cudaMemcpyAsync(h->d_img, d_img, elem_size(img_type) * (size_t)h->W * h->H,
                                      cudaMemcpyDeviceToDevice, h->stream));
        in = h->d_img;
    }
    glsu_dpra::FrameGraph *g = nullptr;
    for (auto &c : h->graphs)
        if (c.exec && c.in == in && c.type == img_type && c.parity == h->phi_parity) g = &c;
    if (!g) {
        g = &h->graphs[h->graph_next];
        h->graph_next = (h->graph_next + 1) % 4;
        if (g->exec) cudaGraphExecDestroy(g->exec);
        *g = glsu_dpra::FrameGraph();
        GLSU_CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = dpra_enqueue_frame(h, in, img_type);
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
        if (rc != GLSU_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture of a frame");
        cudaGraphExec_t exec = nullptr;
        const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return cuda_fail(ie, "cudaGraphInstantiate of a frame");
        g->in = in;
        g->type = img_type;
        g->parity = h->phi_parity;
        g->exec = exec;
    }
    GLSU_CUDA_TRY(cudaGraphLaunch(g->exec, h->stream));
    return GLSU_OK;
}

extern "C" int glsu_dpra_set_graph(glsu_dpra *h, int enable)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    GLSU_CUDA_TRY(cudaStreamSynchronize(h->stream));
    dpra_drop_graphs(h);
    h->use_graph = enable != 0;
    return GLSU_OK;
}

extern "C" int glsu_dpra_per_frame_device(glsu_dpra *h, const void *d_img, int img_type, void *d_dphi)
{
    if (!h || !d_img) return fail(GLSU_ERR_INVALID, "null argument");
    GLSU_TRY(dpra_check_type(h, img_type));
    // The first frame after a configuration change runs eagerly, so that
    // one-time host work (kernel attributes, the automatic threshold) stays
    // out of the capture; the legacy default stream cannot be captured.
    if (h->use_graph && !h->timing && h->graph_warm && h->stream) {
        GLSU_TRY(dpra_graph_frame(h, d_img, img_type));
    } else {
        GLSU_TRY(dpra_enqueue_frame(h, d_img, img_type));
        h->graph_warm = true;
    }
    h->synced = false;
    h->frames_done++;
    if (d_dphi) {
        const size_t es = h->prec == GLSU_F32 ? 4 : 8;
        GLSU_CUDA_TRY(cudaMemcpyAsync(d_dphi, h->d_phi[GLSU_DPHI], es * (size_t)h->W * h->H,
                                      cudaMemcpyDeviceToDevice, h->stream));
    }
    return GLSU_OK;
}

extern "C" int glsu_dpra_per_frame(glsu_dpra *h, const void *h_img, int img_type, void *h_dphi, double *time_ms)
{
    if (!h || !h_img || !h_dphi) return fail(GLSU_ERR_INVALID, "null argument");
    GLSU_TRY(dpra_check_type(h, img_type));
    const size_t N = (size_t)h->W * h->H;
    const size_t in_bytes = elem_size(img_type) * N;
    const size_t es = h->prec == GLSU_F32 ? 4 : 8;
    const bool pin_in = is_pinned(h_img), pin_out = is_pinned(h_dphi);
    if (!pin_in) std::memcpy(h->h_in, h_img, in_bytes);
    GLSU_CUDA_TRY(cudaEventRecord(h->t0, h->stream));
    GLSU_CUDA_TRY(cudaMemcpyAsync(h->d_img, pin_in ? h_img : h->h_in, in_bytes, cudaMemcpyHostToDevice, h->stream));
    GLSU_TRY(glsu_dpra_per_frame_device(h, h->d_img, img_type, nullptr));
    GLSU_CUDA_TRY(cudaMemcpyAsync(pin_out ? h_dphi : h->h_out, h->d_phi[GLSU_DPHI], es * N, cudaMemcpyDeviceToHost,
                                  h->stream));
    GLSU_CUDA_TRY(cudaEventRecord(h->t1, h->stream));
    GLSU_TRY(h->wff.check_device_error(h->stream));
    if (h->sur) GLSU_TRY(h->sur->check_error());
    if (!pin_out) std::memcpy(h_dphi, h->h_out, es * N);
    if (time_ms) {
        float ms = 0;
        GLSU_CUDA_TRY(cudaEventElapsedTime(&ms, h->t0, h->t1));
        *time_ms = ms;
    }
    return GLSU_OK;
}

extern "C" int glsu_dpra_update_ref_phi(glsu_dpra *h)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    if (h->synced) return GLSU_OK;  // phi_curr already equals phi_ref
    // The reference copies phi_curr -> phi_ref and dphi -> dphi_ref
    // (DPRA/dpra_cudaf.cu:286-290); exchanging the buffers gives the same
    // state without the copies.
    std::swap(h->d_phi[GLSU_PHI_REF], h->d_phi[GLSU_PHI_CURR]);
    std::swap(h->d_phi[GLSU_DPHI_REF], h->d_phi[GLSU_DPHI]);
    h->phi_parity ^= 1;
    h->synced = true;
    return GLSU_OK;
}

static int dpra_plane(glsu_dpra *h, int which, void **p)
{
    if (which < 0 || which > 3) return fail(GLSU_ERR_INVALID, "bad plane id");
    if (h->synced && which == GLSU_PHI_CURR) which = GLSU_PHI_REF;
    if (h->synced && which == GLSU_DPHI) which = GLSU_DPHI_REF;
    *p = h->d_phi[which];
    return GLSU_OK;
}

extern "C" int glsu_dpra_get(glsu_dpra *h, int which, void *h_out)
{
    if (!h || !h_out) return fail(GLSU_ERR_INVALID, "null argument");
    void *p = nullptr;
    GLSU_TRY(dpra_plane(h, which, &p));
    const size_t es = h->prec == GLSU_F32 ? 4 : 8;
    GLSU_CUDA_TRY(cudaMemcpyAsync(h_out, p, es * (size_t)h->W * h->H, cudaMemcpyDeviceToHost, h->stream));
    GLSU_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return GLSU_OK;
}

extern "C" int glsu_dpra_set_ls_method(glsu_dpra *h, int method)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    dpra_drop_graphs(h);
    if (method != GLSU_LS_FLOAT_FLOAT && method != GLSU_LS_FP64_SUMS)
        return fail(GLSU_ERR_INVALID, "unknown least-squares method");
    h->ls_method = method;
    return GLSU_OK;
}

static const int kLsTiles[3][2] = {{32, 16}, {32, 8}, {32, 32}};

// The float-float tile's shared memory grows with the radius: 32 x 32 does
// not fit at r = 8 (246 KB).
static bool ls_tile_fits(int t, int r)
{
    const int lim = device_smem_optin();
    return lim > 0 && dpra_ls_ff_smem(kLsTiles[t][0], kLsTiles[t][1], r) <= (size_t)lim;
}

extern "C" int glsu_dpra_set_ls_tile(glsu_dpra *h, int tile_width, int tile_height)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    for (int t = 0; t < 3; t++)
        if (kLsTiles[t][0] == tile_width && kLsTiles[t][1] == tile_height) {
            if (!ls_tile_fits(t, h->r))
                return fail(GLSU_ERR_UNSUPPORTED,
                            "a " + std::to_string(tile_width) + "x" + std::to_string(tile_height) +
                                " least-squares tile at radius " + std::to_string(h->r) + " needs " +
                                std::to_string(dpra_ls_ff_smem(tile_width, tile_height, h->r)) +
                                " bytes of shared memory, above the device limit");
            dpra_drop_graphs(h);
            GLSU_CUDA_TRY(cudaStreamSynchronize(h->stream));
            h->ls_tile = t;
            return GLSU_OK;
        }
    return fail(GLSU_ERR_UNSUPPORTED, "least-squares tiles: 32x16, 32x8, 32x32");
}

extern "C" int glsu_dpra_get_ls_tile(const glsu_dpra *h, int *tile_width, int *tile_height)
{
    if (!h || !tile_width || !tile_height) return fail(GLSU_ERR_INVALID, "null argument");
    *tile_width = kLsTiles[h->ls_tile][0];
    *tile_height = kLsTiles[h->ls_tile][1];
    return GLSU_OK;
}

extern "C" int glsu_dpra_tune_ls_tile(glsu_dpra *h, float *ms)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    if (h->prec != GLSU_F32 || h->ls_method != GLSU_LS_FLOAT_FLOAT)
        return fail(GLSU_ERR_UNSUPPORTED, "the least-squares tile is a knob of the FP32 float-float form");
    dpra_drop_graphs(h);
    cudaStream_t s = h->stream;
    // a zero frame against the handle's own reference phase: the kernels'
    // work does not depend on the values
    GLSU_CUDA_TRY(cudaMemsetAsync(h->d_img, 0, (size_t)h->W * h->H * sizeof(float), s));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return fail(GLSU_ERR_CUDA, "cudaEventCreate failed");
    }
    int best = 0, rc = GLSU_OK;
    float best_ms = 0;
    bool any = false;
    for (int t = 0; t < 3 && rc == GLSU_OK; t++) {
        if (!ls_tile_fits(t, h->r)) {  // not a candidate at this radius
            if (ms) ms[t] = -1.f;
            continue;
        }
        for (int k = 0; k < 4 && rc == GLSU_OK; k++) {
            if (k == 1 && cudaEventRecord(e0, s) != cudaSuccess) rc = fail(GLSU_ERR_CUDA, "cudaEventRecord");
            if (rc == GLSU_OK)
                rc = launch_dpra_ls(h->prec, GLSU_F32, h->d_img, h->d_phi[GLSU_PHI_REF], h->d_z, h->W, h->H, h->r, s,
                                    h->ls_method, t);
        }
        float t_ms = 0;
        if (rc == GLSU_OK && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                              cudaEventElapsedTime(&t_ms, e0, e1) != cudaSuccess))
            rc = fail(GLSU_ERR_CUDA, "timing a least-squares tile failed");
        t_ms /= 3;
        if (ms) ms[t] = t_ms;
        if (rc == GLSU_OK && (!any || t_ms < best_ms)) {
            best = t;
            best_ms = t_ms;
            any = true;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != GLSU_OK) return rc;
    h->ls_tile = best;
    return GLSU_OK;
}

extern "C" int glsu_dpra_lsq_device(glsu_dpra *h, void *d_out)
{
    if (!h || !d_out) return fail(GLSU_ERR_INVALID, "null argument");
    const size_t es = h->prec == GLSU_F32 ? 4 : 8;
    GLSU_CUDA_TRY(
        cudaMemcpyAsync(d_out, h->d_z, 2 * es * (size_t)h->W * h->H, cudaMemcpyDeviceToDevice, h->stream));
    return GLSU_OK;
}

extern "C" int glsu_dpra_get_lsq(glsu_dpra *h, void *h_out)
{
    if (!h || !h_out) return fail(GLSU_ERR_INVALID, "null argument");
    const size_t es = h->prec == GLSU_F32 ? 4 : 8;
    GLSU_CUDA_TRY(cudaMemcpyAsync(h_out, h->d_z, 2 * es * (size_t)h->W * h->H, cudaMemcpyDeviceToHost, h->stream));
    GLSU_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return GLSU_OK;
}

extern "C" int glsu_dpra_device_ptr(glsu_dpra *h, int which, void **d_ptr)
{
    if (!h || !d_ptr) return fail(GLSU_ERR_INVALID, "null argument");
    return dpra_plane(h, which, d_ptr);
}

static int dpra_pipeline_init(glsu_dpra *h)
{
    if (h->s_in) return GLSU_OK;
    const size_t N = (size_t)h->W * h->H;
    const size_t es = h->prec == GLSU_F32 ? 4 : 8;
    GLSU_CUDA_TRY(cudaMalloc(&h->d_seq_img1, 8 * N));
    for (int s = 0; s < 2; s++) {
        GLSU_CUDA_TRY(cudaMalloc(&h->d_ring[s], es * N));
        GLSU_CUDA_TRY(cudaEventCreateWithFlags(&h->ev_in[s], cudaEventDisableTiming));
        GLSU_CUDA_TRY(cudaEventCreateWithFlags(&h->ev_comp[s], cudaEventDisableTiming));
        GLSU_CUDA_TRY(cudaEventCreateWithFlags(&h->ev_out[s], cudaEventDisableTiming));
    }
    GLSU_CUDA_TRY(cudaStreamCreateWithFlags(&h->s_out, cudaStreamNonBlocking));
    GLSU_CUDA_TRY(cudaStreamCreateWithFlags(&h->s_in, cudaStreamNonBlocking));  // set last: marks init done
    return GLSU_OK;
}

// Frame loop of DPRA_CPU::operator() (DPRA/dpra_cpu.cpp:58-89) with the
// host<->device copies taken off the compute stream: frame i is uploaded on
// s_in into slot i%2 while frame i-1 computes, and its phase change is copied
// (device to device, on the compute stream) into ring slot i%2 and downloaded
// on s_out while frame i+1 computes.  Slot reuse waits on frame i-2's events.
static int dpra_sequence_pipelined(glsu_dpra *h, int nframes, const char *h_frames, size_t in_bytes,
                                   int img_type, char *h_out, double *time_ms)
{
    GLSU_TRY(dpra_pipeline_init(h));
    const size_t out_bytes = (h->prec == GLSU_F32 ? 4 : 8) * (size_t)h->W * h->H;
    void *d_slot[2] = {h->d_img, h->d_seq_img1};
    GLSU_CUDA_TRY(cudaEventRecord(h->t0, h->stream));
    GLSU_CUDA_TRY(cudaStreamWaitEvent(h->s_in, h->t0, 0));  // earlier work on the compute stream first
    for (int i = 0; i < nframes; i++) {
        const int s = i & 1;
        if (i >= 2) GLSU_CUDA_TRY(cudaStreamWaitEvent(h->s_in, h->ev_comp[s], 0));
        GLSU_CUDA_TRY(cudaMemcpyAsync(d_slot[s], h_frames + in_bytes * i, in_bytes, cudaMemcpyHostToDevice, h->s_in));
        GLSU_CUDA_TRY(cudaEventRecord(h->ev_in[s], h->s_in));
        GLSU_CUDA_TRY(cudaStreamWaitEvent(h->stream, h->ev_in[s], 0));
        if (i >= 2) GLSU_CUDA_TRY(cudaStreamWaitEvent(h->stream, h->ev_out[s], 0));
        GLSU_TRY(glsu_dpra_per_frame_device(h, d_slot[s], img_type, h->d_ring[s]));
        GLSU_CUDA_TRY(cudaEventRecord(h->ev_comp[s], h->stream));
        GLSU_CUDA_TRY(cudaStreamWaitEvent(h->s_out, h->ev_comp[s], 0));
        GLSU_CUDA_TRY(cudaMemcpyAsync(h_out + out_bytes * i, h->d_ring[s], out_bytes, cudaMemcpyDeviceToHost, h->s_out));
        GLSU_CUDA_TRY(cudaEventRecord(h->ev_out[s], h->s_out));
        if (i % h->rr == 0) GLSU_TRY(glsu_dpra_update_ref_phi(h));
    }
    // the compute stream is done with the last frame once s_out has its copy
    GLSU_CUDA_TRY(cudaEventRecord(h->t1, h->s_out));
    GLSU_CUDA_TRY(cudaStreamWaitEvent(h->stream, h->t1, 0));
    GLSU_TRY(h->wff.check_device_error(h->stream));
    if (h->sur) GLSU_TRY(h->sur->check_error());
    GLSU_CUDA_TRY(cudaEventSynchronize(h->t1));
    if (time_ms) {
        float ms = 0;
        GLSU_CUDA_TRY(cudaEventElapsedTime(&ms, h->t0, h->t1));
        *time_ms = ms;
    }
    return GLSU_OK;
}

extern "C" int glsu_dpra_sequence(glsu_dpra *h, int nframes, const void *h_frames, int img_type, void *h_dphi_all,
                                  double *time_ms)
{
    if (!h || !h_frames || !h_dphi_all || nframes < 0) return fail(GLSU_ERR_INVALID, "bad argument");
    GLSU_TRY(dpra_check_type(h, img_type));
    const size_t N = (size_t)h->W * h->H;
    const size_t es = h->prec == GLSU_F32 ? 4 : 8;
    if (nframes > 0 && is_pinned(h_frames) && is_pinned(h_dphi_all) &&
        is_pinned((const char *)h_frames + elem_size(img_type) * N * nframes - 1) &&
        is_pinned((const char *)h_dphi_all + es * N * nframes - 1))
        return dpra_sequence_pipelined(h, nframes, (const char *)h_frames, elem_size(img_type) * N, img_type,
                                       (char *)h_dphi_all, time_ms);
    double total = 0;
    for (int i = 0; i < nframes; i++) {
        double t = 0;
        GLSU_TRY(glsu_dpra_per_frame(h, (const char *)h_frames + elem_size(img_type) * N * i, img_type,
                                     (char *)h_dphi_all + es * N * i, &t));
        total += t;
        if (i % h->rr == 0) GLSU_TRY(glsu_dpra_update_ref_phi(h));
    }
    if (time_ms) *time_ms = total;
    return GLSU_OK;
}

// Batched form: one frame of each of n independent sequences (handles of any
// sizes, windows and parameters), each enqueued on its handle's own stream so
// that the frames are in flight together; the host returns after
// enqueueing.  Each handle follows the sequence rule: after its i-th batched
// frame the reference is updated when i % rr == 0.
extern "C" int glsu_dpra_batch_step(glsu_dpra *const *handles, int n, const void *const *d_frames, int img_type)
{
    if (!handles || !d_frames || n < 0) return fail(GLSU_ERR_INVALID, "bad argument");
    for (int i = 0; i < n; i++) {
        glsu_dpra *h = handles[i];
        if (!h || !d_frames[i]) continue;  // this sequence has ended
        if (!h->stream) return fail(GLSU_ERR_INVALID, "batched handles need their own streams, not the legacy one");
        for (int j = 0; j < i; j++)
            if (handles[j] == h) return fail(GLSU_ERR_INVALID, "a handle appears twice in one batch step");
        GLSU_TRY(glsu_dpra_per_frame_device(h, d_frames[i], img_type, nullptr));
        if (h->batch_index++ % h->rr == 0) GLSU_TRY(glsu_dpra_update_ref_phi(h));
    }
    return GLSU_OK;
}

// ---------------------------------------------------------------------------
// Staged batch (glsu_dpra_batch_*): one frame of every active sequence per
// step, stage by stage.  Per sequence, on its own stream: the least squares
// and the WFF2 row pass.  Then the FFT column sweeps of all sequences that
// share a transform length as one persistent launch over their work list
// (one launch per length, the lengths on parallel streams); sequences on the
// direct sweep run it on their own stream.  Then per sequence the final row
// pass with the phase update.  The step is captured as one CUDA graph when
// graph mode is on.
// ---------------------------------------------------------------------------
struct glsu_dpra_batch {
    std::vector<glsu_dpra *> h;
    cudaStream_t stream = nullptr;
    std::vector<cudaStream_t> cls_stream;  // one per transform-length class
    std::vector<cudaEvent_t> ev;           // fork/join events
    bool use_graph = false;
    bool warm = false;
    struct Graph {
        std::vector<char> key;
        cudaGraphExec_t exec = nullptr;
    };
    Graph graphs[4];
    int graph_next = 0;
};

static int batch_event(glsu_dpra_batch *b, size_t k, cudaEvent_t *e)
{
    while (b->ev.size() <= k) {
        cudaEvent_t x = nullptr;
        GLSU_CUDA_TRY(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
        b->ev.push_back(x);
    }
    *e = b->ev[k];
    return GLSU_OK;
}

// Enqueue one step on the batch stream for the handles with active[i],
// reading each handle's frame from in[i].
static int batch_enqueue(glsu_dpra_batch *b, const std::vector<char> &active, const std::vector<const void *> &in,
                         int img_type)
{
    size_t ne = 0;
    cudaEvent_t fork = nullptr, e = nullptr;
    GLSU_TRY(batch_event(b, ne++, &fork));
    GLSU_CUDA_TRY(cudaEventRecord(fork, b->stream));
    // stage 1: least squares and row pass (and the direct column sweep)
    std::map<int, std::vector<const WffPlan *>> classes;
    for (size_t i = 0; i < b->h.size(); i++) {
        if (!active[i]) continue;
        glsu_dpra *h = b->h[i];
        GLSU_CUDA_TRY(cudaStreamWaitEvent(h->stream, fork, 0));
        GLSU_TRY(launch_dpra_ls(h->prec, img_type, in[i], h->d_phi[GLSU_PHI_REF], h->d_z, h->W, h->H, h->r,
                                h->stream, h->ls_method, h->ls_tile));
        GLSU_TRY(h->wff.enqueue_pre(h->stream, h->d_z));
        if (h->wff.use_colfft()) classes[h->wff.fft_L].push_back(&h->wff);
        else GLSU_TRY(launch_column_sweep(h->wff, h->stream));
        GLSU_TRY(batch_event(b, ne++, &e));
        GLSU_CUDA_TRY(cudaEventRecord(e, h->stream));
        GLSU_CUDA_TRY(cudaStreamWaitEvent(b->stream, e, 0));
    }
    // stage 2: the FFT column sweeps, one persistent launch per length
    cudaEvent_t pre = nullptr;
    GLSU_TRY(batch_event(b, ne++, &pre));
    GLSU_CUDA_TRY(cudaEventRecord(pre, b->stream));
    size_t c = 0;
    for (auto &kv : classes) {
        if (b->cls_stream.size() <= c) {
            cudaStream_t st = nullptr;
            GLSU_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
            b->cls_stream.push_back(st);
        }
        cudaStream_t st = b->cls_stream[c++];
        GLSU_CUDA_TRY(cudaStreamWaitEvent(st, pre, 0));
        GLSU_TRY(launch_colfft_batch(kv.second.data(), (int)kv.second.size(), st));
        GLSU_TRY(batch_event(b, ne++, &e));
        GLSU_CUDA_TRY(cudaEventRecord(e, st));
        GLSU_CUDA_TRY(cudaStreamWaitEvent(b->stream, e, 0));
    }
    // stage 3: final row pass with the phase update
    cudaEvent_t cols = nullptr;
    GLSU_TRY(batch_event(b, ne++, &cols));
    GLSU_CUDA_TRY(cudaEventRecord(cols, b->stream));
    for (size_t i = 0; i < b->h.size(); i++) {
        if (!active[i]) continue;
        glsu_dpra *h = b->h[i];
        GLSU_CUDA_TRY(cudaStreamWaitEvent(h->stream, cols, 0));
        GLSU_TRY(h->wff.enqueue_final(h->stream, nullptr, h->unwrap ? 2 : 1, h->d_phi[GLSU_PHI_REF],
                                      h->d_phi[GLSU_DPHI_REF], h->d_phi[GLSU_PHI_CURR], h->d_phi[GLSU_DPHI]));
        if (h->unwrap)
            GLSU_TRY(launch_unwrap(h->prec, h->d_phi[GLSU_DPHI], h->d_phi[GLSU_DPHI_REF], h->W, h->H, h->unwrap_row,
                                   h->unwrap_col, h->stream));
        GLSU_TRY(batch_event(b, ne++, &e));
        GLSU_CUDA_TRY(cudaEventRecord(e, h->stream));
        GLSU_CUDA_TRY(cudaStreamWaitEvent(b->stream, e, 0));
    }
    return GLSU_OK;
}

extern "C" int glsu_dpra_batch_create(glsu_dpra_batch **out, glsu_dpra *const *handles, int n)
{
    if (!out || !handles || n < 1) return fail(GLSU_ERR_INVALID, "bad argument");
    *out = nullptr;
    for (int i = 0; i < n; i++) {
        glsu_dpra *h = handles[i];
        if (!h) return fail(GLSU_ERR_INVALID, "null handle");
        if (h->prec != GLSU_F32 || h->sur)
            return fail(GLSU_ERR_UNSUPPORTED, "the staged batch runs FP32 handles in the plain form");
        if (!h->stream) return fail(GLSU_ERR_INVALID, "batched handles need their own streams, not the legacy one");
        for (int j = 0; j < i; j++)
            if (handles[j] == h) return fail(GLSU_ERR_INVALID, "a handle appears twice in one batch");
    }
    glsu_dpra_batch *b = new glsu_dpra_batch();
    b->h.assign(handles, handles + n);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        return fail(GLSU_ERR_CUDA, "cudaStreamCreate failed");
    }
    *out = b;
    return GLSU_OK;
}

static void batch_drop_graphs(glsu_dpra_batch *b)
{
    for (auto &g : b->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = glsu_dpra_batch::Graph();
    }
    b->warm = false;
}

extern "C" int glsu_dpra_batch_destroy(glsu_dpra_batch *b)
{
    if (!b) return GLSU_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    batch_drop_graphs(b);
    for (auto st : b->cls_stream) cudaStreamDestroy(st);
    for (auto e : b->ev) cudaEventDestroy(e);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return GLSU_OK;
}

extern "C" int glsu_dpra_batch_set_graph(glsu_dpra_batch *b, int enable)
{
    if (!b) return fail(GLSU_ERR_INVALID, "null batch");
    GLSU_CUDA_TRY(cudaStreamSynchronize(b->stream));
    batch_drop_graphs(b);
    b->use_graph = enable != 0;
    return GLSU_OK;
}

extern "C" int glsu_dpra_batch_run(glsu_dpra_batch *b, const void *const *d_frames, int img_type)
{
    if (!b || !d_frames) return fail(GLSU_ERR_INVALID, "null argument");
    const size_t n = b->h.size();
    std::vector<char> active(n, 0);
    std::vector<const void *> in(n, nullptr);
    for (size_t i = 0; i < n; i++) {
        if (!d_frames[i]) continue;  // this sequence has ended
        GLSU_TRY(dpra_check_type(b->h[i], img_type));
        if (img_type == GLSU_F64) return fail(GLSU_ERR_INVALID, "FP32 handles take U8 or F32 frames");
        active[i] = 1;
        in[i] = d_frames[i];
    }
    if (b->use_graph && b->warm) {
        // the graph reads each handle's own frame buffer: copy the inputs in
        std::vector<char> key(active);
        key.push_back((char)img_type);
        for (size_t i = 0; i < n; i++) {
            glsu_dpra *h = b->h[i];
            key.push_back((char)h->phi_parity);
            if (!active[i]) continue;
            GLSU_CUDA_TRY(cudaMemcpyAsync(h->d_img, d_frames[i], elem_size(img_type) * (size_t)h->W * h->H,
                                          cudaMemcpyDeviceToDevice, b->stream));
            in[i] = h->d_img;
        }
        glsu_dpra_batch::Graph *g = nullptr;
        for (auto &c : b->graphs)
            if (c.exec && c.key == key) g = &c;
        if (!g) {
            g = &b->graphs[b->graph_next];
            b->graph_next = (b->graph_next + 1) % 4;
            if (g->exec) cudaGraphExecDestroy(g->exec);
            *g = glsu_dpra_batch::Graph();
            GLSU_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            const int rc = batch_enqueue(b, active, in, img_type);
            cudaGraph_t graph = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(b->stream, &graph);
            if (rc != GLSU_OK) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture of a batch step");
            cudaGraphExec_t exec = nullptr;
            const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (ie != cudaSuccess) return cuda_fail(ie, "cudaGraphInstantiate of a batch step");
            g->key = key;
            g->exec = exec;
        }
        GLSU_CUDA_TRY(cudaGraphLaunch(g->exec, b->stream));
    } else {
        // eager (also the first step: one-time host work stays out of captures)
        GLSU_TRY(batch_enqueue(b, active, in, img_type));
        b->warm = true;
    }
    for (size_t i = 0; i < n; i++) {
        if (!active[i]) continue;
        glsu_dpra *h = b->h[i];
        h->synced = false;
        h->frames_done++;
        if (h->batch_index++ % h->rr == 0) GLSU_TRY(glsu_dpra_update_ref_phi(h));
    }
    return GLSU_OK;
}

extern "C" int glsu_dpra_batch_sync(glsu_dpra_batch *b)
{
    if (!b) return fail(GLSU_ERR_INVALID, "null batch");
    GLSU_CUDA_TRY(cudaStreamSynchronize(b->stream));
    for (auto h : b->h) GLSU_TRY(h->wff.check_device_error(h->stream));
    return GLSU_OK;
}

extern "C" int glsu_dpra_batch_wait(glsu_dpra *const *handles, int n)
{
    if (!handles || n < 0) return fail(GLSU_ERR_INVALID, "bad argument");
    for (int i = 0; i < n; i++) {
        glsu_dpra *h = handles[i];
        if (!h) continue;
        GLSU_CUDA_TRY(cudaStreamSynchronize(h->stream));
        GLSU_TRY(h->wff.check_device_error(h->stream));
        if (h->sur) GLSU_TRY(h->sur->check_error());
    }
    return GLSU_OK;
}

extern "C" int glsu_dpra_set_unwrap(glsu_dpra *h, int enable, int start_row, int start_col)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    dpra_drop_graphs(h);
    if (start_row >= h->H || start_col >= h->W) return fail(GLSU_ERR_INVALID, "unwrap start outside the image");
    if (h->W > 4096 || h->H > 4096) return fail(GLSU_ERR_UNSUPPORTED, "unwrap supports sides up to 4096");
    h->unwrap = enable != 0;
    h->unwrap_row = start_row;
    h->unwrap_col = start_col;
    return GLSU_OK;
}

extern "C" int glsu_unwrap2_device(int precision, void *d_p, int width, int height, int start_row, int start_col,
                                   void *cuda_stream)
{
    if (!d_p) return fail(GLSU_ERR_INVALID, "null argument");
    return launch_unwrap(precision, d_p, nullptr, width, height, start_row, start_col, (cudaStream_t)cuda_stream);
}

extern "C" int glsu_dpra_stage_timing(glsu_dpra *h, int enable)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    dpra_drop_graphs(h);
    h->timing = enable != 0;
    return GLSU_OK;
}

extern "C" int glsu_dpra_stage_times(glsu_dpra *h, float *ms, int n)
{
    if (!h || !ms) return fail(GLSU_ERR_INVALID, "null argument");
    if (!h->timing || h->frames_done == 0) return 0;
    GLSU_CUDA_TRY(cudaStreamSynchronize(h->stream));
    const cudaEvent_t seq[5] = {h->ev[4], h->ev[0], h->ev[1], h->ev[2], h->ev[3]};
    int k = 0;
    for (; k < 4 && k < n; k++) GLSU_CUDA_TRY(cudaEventElapsedTime(&ms[k], seq[k], seq[k + 1]));
    if (!h->sur) return k;
    // surrogate form: the network split into layer 0, layers 1-6, layer 7
    const cudaEvent_t net[4] = {h->ev[0], h->ev[6], h->ev[7], h->ev[1]};
    for (int j = 0; j < 3 && k < n; j++, k++) GLSU_CUDA_TRY(cudaEventElapsedTime(&ms[k], net[j], net[j + 1]));
    // and the probe sweep on its own (beside the network when overlapped)
    if (k < n && h->sur_tol > 0) {
        GLSU_CUDA_TRY(cudaStreamSynchronize(h->s_probe));
        GLSU_CUDA_TRY(cudaEventElapsedTime(&ms[k], h->ev_p[0], h->ev_p[1]));
        k++;
    }
    return k;
}

// ===========================================================================
// AIA
// ===========================================================================
extern "C" int glsu_aia_create(glsu_aia **out, int M, int cols, int rows)
{
    if (!out) return fail(GLSU_ERR_INVALID, "null handle pointer");
    *out = nullptr;
    if (M < 3 || M > 32) return fail(GLSU_ERR_INVALID, "AIA needs 3..32 frames");
    if (cols < 1 || rows < 1) return fail(GLSU_ERR_INVALID, "image size must be positive");
    glsu_aia *h = new glsu_aia();
    h->M = M;
    h->cols = cols;
    h->rows = rows;
    h->N = cols * rows;
    int rc = wff_setup_stream(&h->stream, &h->own_stream);
    h->dev.M = M;
    h->dev.N = h->N;
    h->dev.nblocks = 152 * 2;
    if (rc == GLSU_OK) {
        const size_t nv = 5 + 3 * (size_t)M;
        bool ok = cudaMalloc(&h->d_frames, (size_t)M * h->N * 4) == cudaSuccess &&
                  cudaMalloc((void **)&h->d_phi, sizeof(float) * h->N) == cudaSuccess &&
                  cudaMalloc((void **)&h->dev.d_part, sizeof(double) * nv * h->dev.nblocks) == cudaSuccess &&
                  cudaMalloc((void **)&h->dev.d_state, sizeof(double) * (2 * M + 3)) == cudaSuccess &&
                  cudaMalloc((void **)&h->dev.d_done, sizeof(int)) == cudaSuccess;
        if (!ok) rc = fail(GLSU_ERR_ALLOC, "AIA buffer allocation failed");
    }
    if (rc == GLSU_OK && (cudaEventCreate(&h->t0) != cudaSuccess || cudaEventCreate(&h->t1) != cudaSuccess))
        rc = fail(GLSU_ERR_CUDA, "cudaEventCreate failed");
    if (rc != GLSU_OK) {
        glsu_aia_destroy(h);
        return rc;
    }
    *out = h;
    return GLSU_OK;
}

extern "C" int glsu_aia_destroy(glsu_aia *h)
{
    if (!h) return GLSU_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->d_frames);
    cudaFree(h->d_phi);
    cudaFree(h->dev.d_part);
    cudaFree(h->dev.d_state);
    cudaFree(h->dev.d_done);
    if (h->t0) cudaEventDestroy(h->t0);
    if (h->t1) cudaEventDestroy(h->t1);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return GLSU_OK;
}

extern "C" int glsu_aia_set_stream(glsu_aia *h, void *stream)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    if (h->own_stream && h->stream) {
        cudaStreamSynchronize(h->stream);
        cudaStreamDestroy(h->stream);
    }
    h->stream = (cudaStream_t)stream;
    h->own_stream = false;
    return GLSU_OK;
}

static int aia_core(glsu_aia *h, const void *d_frames, int img_type, float *d_phi, float *h_deltas, int n_deltas_in,
                    int *iters, float *err, int max_iter, float max_err, uint64_t seed, double *time_ms)
{
    std::vector<float> d0(h->M);
    if (n_deltas_in == h->M) {
        for (int i = 0; i < h->M; i++) d0[i] = h_deltas[i];
    } else {
        GLSU_TRY(glsu_aia_random_deltas(h->M, seed, d0.data()));
    }
    std::vector<double> dd(d0.begin(), d0.end());
    cudaStream_t s = h->stream;
    GLSU_CUDA_TRY(cudaEventRecord(h->t0, s));
    GLSU_TRY(aia_launch_init(h->dev, dd.data(), s));
    for (int it = 0; it < max_iter; it++) {
        GLSU_TRY(aia_launch_pass(h->dev, img_type, d_frames, 0, nullptr, s));
        GLSU_TRY(aia_launch_solve(h->dev, max_iter, (double)max_err, s));
    }
    GLSU_CUDA_TRY(cudaEventRecord(h->t1, s));
    GLSU_TRY(aia_launch_pass(h->dev, img_type, d_frames, 1, d_phi, s));
    GLSU_TRY(aia_launch_finalize(h->dev, d_phi, s));
    std::vector<double> st(2 * h->M + 3);
    GLSU_CUDA_TRY(cudaMemcpyAsync(st.data(), h->dev.d_state, sizeof(double) * st.size(), cudaMemcpyDeviceToHost, s));
    GLSU_CUDA_TRY(cudaStreamSynchronize(s));
    if (st[2 * h->M + 2] != 0) return fail(GLSU_ERR_NOT_POSDEF, "The leading minor is not positive definite");
    for (int i = 0; i < h->M; i++) h_deltas[i] = (float)st[i];
    if (iters) *iters = (int)st[2 * h->M + 1];
    if (err) *err = max_iter > 0 ? (float)st[2 * h->M] : 2.0f * max_err;
    if (time_ms) {
        float ms = 0;
        GLSU_CUDA_TRY(cudaEventElapsedTime(&ms, h->t0, h->t1));
        *time_ms = ms;
    }
    return GLSU_OK;
}

extern "C" int glsu_aia_set_convergence(glsu_aia *h, int mode)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    if (mode != GLSU_AIA_ERR_ABS && mode != GLSU_AIA_ERR_RELATIVE)
        return fail(GLSU_ERR_INVALID, "unknown AIA convergence measure");
    h->dev.err_mode = mode;
    return GLSU_OK;
}

extern "C" int glsu_aia_run(glsu_aia *h, const void *const *h_frames, int img_type, float *h_phi, float *h_deltas,
                            int n_deltas_in, double *time_ms, int *iters, float *err, int max_iter, float max_err,
                            uint64_t seed)
{
    if (!h || !h_frames || !h_phi || !h_deltas) return fail(GLSU_ERR_INVALID, "null argument");
    if (img_type != GLSU_U8 && img_type != GLSU_F32) return fail(GLSU_ERR_INVALID, "frames must be U8 or F32");
    const size_t fb = elem_size(img_type) * (size_t)h->N;
    for (int i = 0; i < h->M; i++) {
        if (!h_frames[i]) return fail(GLSU_ERR_INVALID, "null frame");
        GLSU_CUDA_TRY(cudaMemcpyAsync((char *)h->d_frames + fb * i, h_frames[i], fb, cudaMemcpyHostToDevice, h->stream));
    }
    GLSU_TRY(aia_core(h, h->d_frames, img_type, h->d_phi, h_deltas, n_deltas_in, iters, err, max_iter, max_err, seed,
                      time_ms));
    GLSU_CUDA_TRY(cudaMemcpy(h_phi, h->d_phi, sizeof(float) * h->N, cudaMemcpyDeviceToHost));
    return GLSU_OK;
}

extern "C" int glsu_aia_run_device(glsu_aia *h, const void *d_frames, int img_type, float *d_phi, float *h_deltas,
                                   int n_deltas_in, int *iters, float *err, int max_iter, float max_err,
                                   uint64_t seed)
{
    if (!h || !d_frames || !d_phi || !h_deltas) return fail(GLSU_ERR_INVALID, "null argument");
    if (img_type != GLSU_U8 && img_type != GLSU_F32) return fail(GLSU_ERR_INVALID, "frames must be U8 or F32");
    return aia_core(h, d_frames, img_type, d_phi, h_deltas, n_deltas_in, iters, err, max_iter, max_err, seed,
                    nullptr);
}
