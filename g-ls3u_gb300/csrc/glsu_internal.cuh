// glsu_internal.cuh -- shared declarations of the G-LS3U CUDA library (sm_103a).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/glsu.h"

namespace glsu {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define GLSU_CUDA_TRY(call)                                  \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);  \
    } while (0)

#define GLSU_TRY(call)                  \
    do {                                \
        int rc_ = (call);               \
        if (rc_ != GLSU_OK) return rc_; \
    } while (0)

// Raise the dynamic shared-memory limit of kernel `func` to `bytes` on the
// current device, once per (kernel, device), thread-safe.  carveout >= 0 also
// sets the kernel's preferred shared-memory carveout (percent).
int raise_smem_limit(const void *func, int bytes, int carveout = -1);
// Multiprocessor count of the current device (looked up once per device).
int device_sm_count();
// Largest dynamic shared memory a block may opt into on the current device (0 if unknown).
int device_smem_optin();
// Dynamic shared memory of the float-float least squares with a tx x ty tile at radius r.
size_t dpra_ls_ff_smem(int tx, int ty, int r);

// ---------------------------------------------------------------------------
// complex element types
// ---------------------------------------------------------------------------
template <typename T> struct C2T;
template <> struct C2T<float> { using type = float2; };
template <> struct C2T<double> { using type = double2; };
template <typename T> using C2 = typename C2T<T>::type;

// Largest supported window half-size round(3*sigma) of WFF2.  Kernels are
// instantiated for half-sizes 12, 20, 30, 45 and 60; a smaller half-size
// runs in the next instantiation with zero taps outside its window, which
// leaves every sum unchanged.
constexpr int kMaxHalf = 60;
int instantiated_half(int s);  // -> 12/20/30/45/60, or -1 when s > kMaxHalf

// Padding (in elements) of the phasor tables on each side.
constexpr int kPhasorPad = 2 * kMaxHalf;

// Bounded device-side waits: spin limit of an mbarrier wait before the
// kernel records GLSU_ERR_TIMEOUT in its error word and returns.
constexpr long long kSpinLimit = 1ll << 26;

// Blocks (and partial sums) of the automatic-threshold reduction.
constexpr int kThrBlocks = 304;

// Tiles of a frame that the plain WFF2 recomputes (surrogate fallback).
// With flags set, each WFF2 kernel CTA runs only when its output rectangle,
// grown by (my, mx), meets a flagged tile, and the final pass writes only
// pixels of flagged tiles.  The image border (crop) stays the full frame's.
struct TileMask {
    const int *flags = nullptr;  // [nty][ntx], nonzero = recompute
    int tile = 0, ntx = 0, nty = 0;
    int my = 0, mx = 0;  // margins of the kernel being launched
    __device__ __forceinline__ bool any(int y0, int y1, int x0, int x1) const
    {
        const int ty0 = max(0, y0 - my) / tile, ty1 = min(nty - 1, (y1 - 1 + my) / tile);
        const int tx0 = max(0, x0 - mx) / tile, tx1 = min(ntx - 1, (x1 - 1 + mx) / tile);
        for (int ty = ty0; ty <= ty1; ty++)
            for (int tx = tx0; tx <= tx1; tx++)
                if (flags[ty * ntx + tx]) return true;
        return false;
    }
    __device__ __forceinline__ bool at(int y, int x) const { return flags[(y / tile) * ntx + x / tile] != 0; }
};

// Exact sparse WFF2 probe: per tile one P x P patch, P = 8 for window
// half-sizes (instantiated) up to 20, 4 above (P <= kProbeMaxP).
constexpr int kProbeMaxP = 8;
int probe_patch_for_half(int s_inst);
// complex elements of the probe's row-pass block of one (tile, wx)
size_t probe_rows_elems(int s_inst);
struct ProbeOut {
    float2 *partial = nullptr;  // [ntiles][nfx * parts][P*P] partial sums
    int2 *sites = nullptr;      // [ntiles] (row, col) of each patch
    float *resid = nullptr;     // [ntiles] RMS phase residual of the surrogate
    int *flags = nullptr;       // [ntiles] residual > tolerance
    int *counts = nullptr;      // [2] cumulative: tiles probed, tiles flagged
    float2 *rows = nullptr;     // [ntiles][nfx][probe_rows_elems]: row-filtered input of each (tile, wx)
    uint32_t *seed = nullptr;   // frame counter on the device: the patch positions' hash seed (null: the
                                // seed argument of the sweep)
};

// ---------------------------------------------------------------------------
// WFF2 plan: the frequency sweep on the device (see wff_kernels.cu)
// ---------------------------------------------------------------------------
struct WffPlan {
    int prec = GLSU_F32;
    int W = 0, H = 0, pitch = 0;  // pitch: row pitch (elements) of the internal planes
    glsu_wff_params p{};
    int sx = 0, sy = 0;          // true half window sizes
    int sxi = 0, syi = 0;        // instantiated half sizes
    int nfx = 0, nfy = 0;        // frequency counts
    int Wp = 0, Hp = 0;          // FFT-padded plane of the reference formulation
    double thr_host = -1;        // threshold in use (after the first run when automatic)
    bool thr_ready = false;

    // device buffers
    void *d_ex = nullptr;   // nfx x (pitch + 2*pad) phasors exp(-j wx x)
    void *d_ey = nullptr;   // nfy x (H + 2*pad)     phasors exp(-j wy y)
    void *d_R = nullptr;    // nfx planes H x pitch: row-filtered, demodulated input
    void *d_C = nullptr;    // nfx planes H x pitch: column sweep output
    void *d_thr = nullptr;  // 1 element of T: threshold used by the kernels
    double *d_part = nullptr;  // partial sums of the automatic threshold
    int *d_err = nullptr;      // device error word (bounded waits)
    CUtensorMap tmR;        // TMA descriptor of d_R (3D: 2*pitch floats x H x nfx)
    bool external_scratch = false;  // d_R/d_C/d_thr/d_part/d_err owned elsewhere

    // host copies of the taps (device code receives them as kernel parameters)
    double gx[2 * kMaxHalf + 1], gy[2 * kMaxHalf + 1];
    double inv_norm = 1, scale = 1;

    int init(int precision, int width, int height, const glsu_wff_params &prm);
    int alloc_device();
    int upload_tables(cudaStream_t s);
    int make_tensor_map();
    void release();
    size_t plane_bytes() const;  // bytes of one internal plane
    // Enqueue one WFF2 of d_f (H x W complex).  final_mode 0 writes the
    // filtered field to d_out; final_mode 1 applies the DPRA phase update
    // instead (phi_ref, dphi_ref -> phi_curr, dphi).
    int enqueue(cudaStream_t s, const void *d_f, void *d_out, int final_mode, const void *phi_ref,
                const void *dphi_ref, void *phi_curr, void *dphi, cudaEvent_t *stage_ev);
    // Only the row pass of d_f into the R planes (whole frame, no tile mask).
    int enqueue_rows(cudaStream_t s, const void *d_f);
    // The stages of enqueue one at a time (whole frame): the threshold and
    // the row pass; the column sweep (launch_column_sweep); the final row
    // pass with final_mode as in enqueue.
    int enqueue_pre(cudaStream_t s, const void *d_f);
    int enqueue_final(cudaStream_t s, void *d_out, int final_mode, const void *phi_ref, const void *dphi_ref,
                      void *phi_curr, void *dphi);
    int check_device_error(cudaStream_t s);

    // Tile mask of the next enqueue (flags == nullptr: whole frame), and the
    // device list of column tiles a masked run needs (alloc_tile_list).
    TileMask mask;
    int2 *d_list = nullptr;
    int *d_list_count = nullptr;
    int alloc_tile_list();
    // Ensure the threshold on the device (automatic: from d_f, once).
    int ensure_threshold(cudaStream_t s, const void *d_f);
    // FP32 only, half-sizes up to 45: exact WFF2 of d_f on one P x P patch per tile (patch
    // position hashed from seed and the tile), compared with d_cmp (complex,
    // the surrogate's output): RMS phase residual over patch pixels with
    // |WFF2| >= 0.1, flag when above tol.
    int enqueue_probe(cudaStream_t s, const void *d_f, const void *d_cmp, int tile, int P, uint32_t seed,
                      double tol, const ProbeOut &o);
    // The same in two parts: the exact patches (row and column passes) on
    // one stream, then the residuals and flags (after the sweep, e.g. on
    // another stream behind an event).
    int enqueue_probe_sweep(cudaStream_t s, const void *d_f, int tile, int P, uint32_t seed, const ProbeOut &o);
    int enqueue_probe_resid(cudaStream_t s, const void *d_cmp, double tol, const ProbeOut &o);
    int probe_parts = 0, probe_P = 0, probe_ntiles = 0;  // set by the last sweep

    // Column sweep by shared-memory FFTs (FP32 form; see wff_colfft.cu).
    int method = GLSU_METHOD_AUTO;  // GLSU_METHOD_AUTO / DIRECT / FFT
    int fft_L = 0, fft_nst = 0;     // fft_L == 0: no FFT plan, the direct kernel runs
    int fft_radix[12];
    int fft_nc = 0;                 // columns per CTA of the FFT sweep (4 or 2)
    int fft_order = 0;              // radix order of the stages (see fft_factor)
    void *d_khat = nullptr;         // nfy x fft_L spectra of the modulated windows
    void *d_tw = nullptr;           // fft_L twiddles e^{-2 pi i t / L}
    int init_colfft();
    int build_colfft(int L);  // tables for transform length L, default plan variant
    void release_colfft();
    // FFT plan variant: nc columns per CTA, radix order; GLSU_ERR_UNSUPPORTED
    // where it does not fit (the plan is then unchanged).
    int set_fft_plan(int nc, int order);

    // Autotuner (wff_colfft.cu): with GLSU_METHOD_AUTO the column sweep is
    // chosen from the shape by a cost model (deterministic); with
    // GLSU_METHOD_TIMED it is the candidate (direct kernel or FFT plan
    // variant) measured fastest for this shape, timed once per shape and
    // process.
    bool tuned = false;
    bool timed = false;  // the last resolution was by timing
    int auto_method = GLSU_METHOD_DIRECT;
    float tune_ms_direct = 0, tune_ms_fft = 0;
    int autotune(cudaStream_t s);
    int choose_by_model();
    double model_ms(int method) const;
    int column_method() const
    {
        return (method == GLSU_METHOD_AUTO || method == GLSU_METHOD_TIMED) ? auto_method : method;
    }
    bool use_colfft() const { return fft_L > 0 && d_khat != nullptr && column_method() == GLSU_METHOD_FFT; }
};

// The transform lengths the autotuner times for this plan (cheapest first).
int fft_length_candidates(const WffPlan &P, int *out, int n);
// The column sweep of a full-frame run (FFT or direct, as the plan selects).
int launch_column_sweep(WffPlan &P, cudaStream_t s);

int launch_colfft(const WffPlan &P, cudaStream_t s);
// The FFT column sweep of n plans of one transform length (each running the
// FFT sweep, no tile mask) as one persistent launch over their work list.
int launch_colfft_batch(const WffPlan *const *plans, int n, cudaStream_t s);
// Compact the ncx x ncy tiles (ty_rows x tx_cols outputs each) of a column
// sweep that a masked run needs into list / *count (device, index order).
int launch_mask_list(const TileMask &m, int ncx, int ncy, int ty_rows, int tx_cols, int2 *list, int *count,
                     cudaStream_t s);

// ---------------------------------------------------------------------------
// kernel launchers
// ---------------------------------------------------------------------------
// tile (FP32 float-float form only): 0 = 32 x 16 outputs per CTA (the
// default), 1 = 32 x 8, 2 = 32 x 32.
int launch_dpra_ls(int prec, int img_type, const void *d_img, const void *d_phiref, void *d_z, int W, int H,
                   int r, cudaStream_t s, int method = GLSU_LS_FLOAT_FLOAT, int tile = 0);
int launch_dpra_update(int prec, const void *d_filtered, const void *phiref, const void *dphiref,
                       void *phicurr, void *dphi, int n, cudaStream_t s);
// Line-scanning unwrapping in place; d_add (optional) is added to every
// element; negative starts select MATLAB's default (the image centre).
int launch_unwrap(int prec, void *d_p, const void *d_add, int W, int H, int row0, int col0, cudaStream_t s);

// Surrogate network (sur_kernels.cu).  FP32 master parameters, per layer
// W[co][ci][3][3] then b[co]: layer 0 (2 -> 32), layers 1..6 (32 -> 32),
// layer 7 (32 -> 2).
constexpr int kSurLayers = 8;
constexpr int kSurL0Params = 32 * 2 * 9 + 32;
constexpr int kSurL32Params = 32 * 32 * 9 + 32;
constexpr int kSurL7Params = 2 * 32 * 9 + 2;
constexpr int kSurParams = kSurL0Params + 6 * kSurL32Params + kSurL7Params;
inline int sur_layer_offset(int l) { return l == 0 ? 0 : kSurL0Params + (l - 1) * kSurL32Params; }

struct SurConvArgs {
    int B = 0, H = 0, W = 0, dil = 1;
    const uint16_t *wpack = nullptr;  // packed BF16 B operand of the layer
    const float *bias = nullptr;      // [32] (hidden layer) / [2] (last layer) or null
    const uint16_t *mask = nullptr;   // [B][H][W][32]: output zeroed where mask <= 0 (null: none)
    uint16_t *out = nullptr;          // hidden layer: [B][H][W][32] BF16
    int relu = 1;
    int *err = nullptr;
    // last layer: y = z + conv + bias; cout = y / |y| (inference) or yout = y (training)
    const float2 *z = nullptr;
    float2 *cout = nullptr, *yout = nullptr;
    int max_ctas_per_sm = 0;  // 0: as many as fit; else a cap (room for a concurrent kernel)
};
// Weights of the first (CUDA-core) layer, passed to its kernel by value
// (a shared-memory copy read once per FMA made it load-bound).
struct SurL0W {
    float w[32 * 18];  // [co][ci][t], BF16-rounded
    float b[32];
};
int sur_make_map(CUtensorMap *tm, const void *act, int B, int H, int W, int dil);
int sur_make_out_map(CUtensorMap *tm, const void *act, int B, int H, int W);

// ---------------------------------------------------------------------------
// WFR2 (wfr_kernels.cu): per-wx partial arg-max planes and curvature scratch
// ---------------------------------------------------------------------------
struct WfrBuffers {
    void *pabs = nullptr;  // [nfx][H][W] T: best |sf| over wy
    int *pk = nullptr;     // [nfx][H][W]: its wy index
    void *pph = nullptr;   // [nfx][H][W] T: its angle(sf)
    void *A = nullptr, *B = nullptr;  // H x W T: row pass of the curvature convolutions
    int alloc(const WffPlan &P);
    void release();
};
// Enqueue one WFR2 of d_f (H x W complex) into the eight result maps.
int enqueue_wfr(WffPlan &P, const WfrBuffers &wb, cudaStream_t s, const void *d_f, const glsu_wfr_results &z);
int launch_sur_conv(const CUtensorMap &tm, const CUtensorMap &tmo, const SurConvArgs &a, cudaStream_t s);
// The last layer (32 -> 2, residual, renormalisation) on the tensor cores;
// tm maps its input activation with the layer's dilation.
int launch_sur_last(const CUtensorMap &tm, const SurConvArgs &a, cudaStream_t s);

// AIA
struct AiaDev {
    int M = 0, N = 0;
    int nblocks = 0;
    double *d_part = nullptr;   // nblocks x (5 + 3M) partial sums
    double *d_state = nullptr;  // deltas, old deltas, err, iteration, flags
    int *d_done = nullptr;
    int err_mode = GLSU_AIA_ERR_ABS;  // convergence measure (glsu_aia_set_convergence)
};
int aia_launch_pass(const AiaDev &a, int img_type, const void *d_frames, int final_pass, float *d_phi,
                    cudaStream_t s);
int aia_launch_solve(const AiaDev &a, int max_iter, double max_err, cudaStream_t s);
int aia_launch_init(const AiaDev &a, const double *h_deltas, cudaStream_t s);
int aia_launch_finalize(const AiaDev &a, float *d_phi, cudaStream_t s);

}  // namespace glsu
