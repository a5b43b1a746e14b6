/*
 * glsu.h -- C ABI of the GB300 (sm_103a) G-LS3U hot path.
 *
 * Plain pointers and sizes only.  Every call returns a status code (GLSU_OK or
 * a negative GLSU_ERR_*) and never exits the process; glsu_last_error()
 * returns a message for the calling thread's last failure.  Handles are not
 * thread-safe: use one handle per host thread.  Each handle owns a CUDA
 * stream unless one is set with *_set_stream.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   glsu_wff_*   WFT_FPA::WFT::WFT2_CUDAF / WFT2_CUDA with WFT_TYPE::WFF
 *   glsu_wfr_*   WFT_FPA::WFT::WFT2_CUDAF / WFT2_CUDA with WFT_TYPE::WFR
 *                (WFT/WFT2_CUDAf.h:11-40, WFT/WFT2_CUDA.h), whose CPU twin is
 *                WFT/WFT2_CPU.cpp:190-390
 *   glsu_dpra_*  DPRA::DPRA_CUDAF (DPRA/dpra_cudaf.h:21-46) and the empty
 *                DPRA::DPRA_CUDA (DPRA/dpra_cuda.h:9-14), following the
 *                semantics of DPRA_CPU (DPRA/dpra_cpu.h:30-64)
 *   glsu_aia_*   AIA::AIA_CUDAF (AIA/aia_cudaf.h:15-38)
 * The C++ classes with the reference's names and signatures live in
 * glsu_classes.hpp and are implemented on top of these functions.
 */
#ifndef GLSU_H
#define GLSU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GLSU_OK 0
#define GLSU_ERR_INVALID (-1)     /* bad argument or size                      */
#define GLSU_ERR_PADDING (-2)     /* padded size beyond 4096 (reference: throw -1) */
#define GLSU_ERR_CUDA (-3)        /* a CUDA runtime call failed                */
#define GLSU_ERR_ALLOC (-4)       /* device or pinned allocation failed        */
#define GLSU_ERR_UNSUPPORTED (-5) /* e.g. a window beyond the limits        */
#define GLSU_ERR_NOT_POSDEF (-6)  /* AIA normal matrix not positive definite   */
#define GLSU_ERR_TIMEOUT (-7)     /* a bounded device-side wait gave up        */
#define GLSU_ERR_NO_DEVICE (-8)   /* no CUDA device visible                    */

/* ---- element types ----------------------------------------------------- */
#define GLSU_F32 0 /* float  / float2 complex  (the *_CUDAF classes)        */
#define GLSU_F64 1 /* double / double2 complex (the *_CUDA classes)         */
#define GLSU_U8 2  /* uint8 fringe frames (cv::Mat CV_8UC1 in the reference) */

/* ---- which state plane (glsu_dpra_get / glsu_dpra_device_ptr) ----------- */
#define GLSU_PHI_REF 0
#define GLSU_PHI_CURR 1
#define GLSU_DPHI_REF 2
#define GLSU_DPHI 3

/* Column-sweep method of the WFF2 (glsu_wff_set_method / glsu_dpra_set_method):
 * DIRECT convolves the columns with the truncated window; FFT (FP32 form
 * only) does the same in the frequency domain of each column with
 * shared-memory transforms.  AUTO (the default) picks one of the two from
 * the handle's shape with a cost model of both kernels, so the choice, and
 * therefore every output bit, is the same in every process.  TIMED picks
 * the one measured fastest on this GPU (glsu_wff_tuning); its choice can
 * differ from run to run where the two are close. */
#define GLSU_METHOD_AUTO 0
#define GLSU_METHOD_DIRECT 1
#define GLSU_METHOD_FFT 2
#define GLSU_METHOD_TIMED 3

/* Arithmetic of the FP32 DPRA least squares (glsu_dpra_set_ls_method): the
 * window sums and the solve need more than FP32's 24 bits where phi_ref is
 * locally smooth.  FLOAT_FLOAT forms them in float-float (pairs of FP32,
 * about 48 bits) from FP32 regressors rotated to the tile centre; FP64_SUMS
 * forms them in FP64.  FP64 handles always use FP64. */
#define GLSU_LS_FLOAT_FLOAT 0
#define GLSU_LS_FP64_SUMS 1

/* WFT_TYPE of the reference (WFT-FPA.h enum WFT_TYPE) */
#define GLSU_WFT_WFF 0
#define GLSU_WFT_WFR 1

typedef struct glsu_wff glsu_wff;
typedef struct glsu_dpra glsu_dpra;
typedef struct glsu_aia glsu_aia;

/* WFF2 parameters, in the reference's C++ order: sigma, low, high, step
 * (WFT/WFT2_CUDAf.h:27-33).  thr < 0 selects 6*sqrt(mean(|f|^2)/3), computed
 * on the device at the first call and kept for later calls
 * (WFT/WFT2_CPU.cpp:977-1005). */
typedef struct glsu_wff_params {
    double sigma_x, wxl, wxh, wxi;
    double sigma_y, wyl, wyh, wyi;
    double thr;
} glsu_wff_params;

/* ---- utilities (host only, no device needed) ---------------------------- */
const char *glsu_last_error(void);
int glsu_version(void);
/* Smallest even 2^a3^b5^c7^d size >= x, or -1 (WFT/WFT.h:18-32, WFT/WFT.cpp:10-23). */
int glsu_opt_fft_size(int x);
/* Default WFF/WFR parameters of a WFT_TYPE (WFT/WFT2_CUDAf.cu:852-875). */
int glsu_wft_default_params(int wft_type, glsu_wff_params *p);
/* Parameters DPRA hard-wires for its WFF (DPRA/dpra_cudaf.cu:116-118). */
int glsu_dpra_default_wff_params(glsu_wff_params *p);
/* Number of frequencies on [lo, hi] with step, as the reference computes it
 * in the given precision: int((hi-lo)*(1/step))+1 (WFT/WFT2_CPU.cpp:222-223). */
int glsu_wff_count(double lo, double hi, double step, int precision);
/* Seeded initial AIA phase shifts: d[0]=0, d[1..M-1] ~ N(0,1) (replaces the
 * time-seeded draw of AIA/aia_cpu.cpp:32-46). */
int glsu_aia_random_deltas(int M, uint64_t seed, float *deltas);

/* ---- WFF2: WFT2_CUDAF / WFT2_CUDA with WFT_TYPE::WFF -------------------- */
/* precision: GLSU_F32 or GLSU_F64.  p == NULL: reference WFF defaults.
 * Windows up to half-size round(3*sigma) <= 60 are supported. */
int glsu_wff_create(glsu_wff **out, int precision, int width, int height, const glsu_wff_params *p);
int glsu_wff_destroy(glsu_wff *h);
int glsu_wff_set_stream(glsu_wff *h, void *cuda_stream);
/* d_f: device H*W complex input; d_filtered: device H*W complex output
 * (WFT2_CUDAF::operator(), WFT/WFT2_CUDAf.cu:1003-1011).  Synchronous;
 * *time_ms (may be NULL) receives the device time of the call. */
int glsu_wff_run(glsu_wff *h, const void *d_f, void *d_filtered, double *time_ms);
/* Same, enqueued on the handle's stream without waiting. */
int glsu_wff_run_async(glsu_wff *h, const void *d_f, void *d_filtered);
/* Threshold in use (after the first call when automatic). */
int glsu_wff_threshold(glsu_wff *h, double *thr);
/* Choose the column-sweep method (GLSU_METHOD_*); results agree to FP32
 * rounding.  GLSU_METHOD_FFT fails with GLSU_ERR_UNSUPPORTED where no
 * transform plan exists (FP64 handles). */
int glsu_wff_set_method(glsu_wff *h, int method);
/* Column-sweep autotuner.
 * GLSU_METHOD_AUTO (the default): the FFT sweep at the shortest compiled
 * transform length >= H + 2 sy, with its default CTA width, when the cost
 * model puts it below 0.9 x the direct kernel's time; else the direct
 * kernel.  Decided from the shape only: deterministic.
 * GLSU_METHOD_TIMED: the handle runs the column sweep measured fastest for
 * its shape: the direct kernel, or the FFT sweep at one of the two shortest
 * compiled transform lengths, at either compiled CTA width.  The first
 * handle of a shape in the process times the candidates (a few launches
 * each); later handles of that shape reuse the choice.  The FFT is taken
 * only when at least 10% faster.  GLSU_AUTOTUNE=time in the environment
 * makes AUTO behave as TIMED; GLSU_AUTOTUNE=0 makes both the direct kernel.
 * The methods agree to FP32 rounding, not bit for bit.
 * Compiled transform lengths: 256, 384, 512, 640, 768, 1024, 1280, 1536,
 * 2048, 2560, 3072, 4096 (one radix sequence each, radix order 0); taller
 * windows run the direct kernel. */
typedef struct {
    int method;          /* GLSU_METHOD_DIRECT or GLSU_METHOD_FFT: the sweep that runs */
    int fft_length;      /* transform length of the FFT plan (0: no FFT plan) */
    int fft_columns;     /* columns per CTA of the FFT sweep */
    int fft_radix_order; /* radix order of the FFT passes (always 0) */
    int tuned;           /* 0: not resolved; 1: resolved by timing; 2: by the cost model */
    float ms_direct;     /* column-sweep time of the direct kernel: measured (tuned 1) or modelled (tuned 2) */
    float ms_fft;        /* time of the FFT sweep: best measured (tuned 1) or modelled (tuned 2) */
} glsu_wff_tuning;
int glsu_wff_get_tuning(const glsu_wff *h, glsu_wff_tuning *t);
/* Force an FFT plan variant: columns_per_cta is the length's default
 * (glsu_wff_get_tuning after glsu_wff_set_fft_length) or twice it, and
 * radix_order is 0; GLSU_ERR_UNSUPPORTED otherwise.  Takes effect when the
 * FFT sweep runs. */
int glsu_wff_set_fft_plan(glsu_wff *h, int columns_per_cta, int radix_order);
/* Rebuild the FFT sweep's tables for another compiled transform length
 * (>= H + 2 sy) with its default CTA width. */
int glsu_wff_set_fft_length(glsu_wff *h, int length);
/* The compiled transform lengths >= H + 2 sy, shortest first; returns how
 * many were written (at most n; 0 without an FFT plan). */
int glsu_wff_fft_lengths(const glsu_wff *h, int *lengths, int n);

/* FFT-padded plane of the reference's formulation (kept for API parity). */
int glsu_wff_padded_size(const glsu_wff *h, int *padded_width, int *padded_height);

/* WFF2 in FP32 without allocating any device memory.  This entry point has
 * no counterpart in the reference.  It is for callers that are not allowed
 * to call cudaMalloc: a plugin living inside a host application whose
 * device memory is handed out by that application's own pool, a real-time
 * frame loop that must never stall in the allocator, or a deployment that
 * fixes its whole device-memory budget when the library is loaded.
 *
 * The caller still passes the input d_f and the output d_filtered (device
 * H*W complex64, as glsu_wff_run) and a stream (NULL: the legacy default
 * stream); p == NULL selects the reference WFF defaults.  Scratch comes from
 * one fixed 64 MiB array inside the library, which every GPU that loads the
 * library holds until the process exits; problems whose scratch -- 2 x
 * (number of x-frequencies) planes of H x round_up(W, 128) complex64 plus
 * small tables -- exceeds 64 MiB are rejected with GLSU_ERR_INVALID and a
 * message giving the size needed (256x256 with 21x21 frequencies uses 22 MiB).
 *
 * The first call on a device looks up that array's device address (once
 * per device, with the device current).  Every call blocks until its result
 * is complete: it synchronises the stream to read back the kernels' error
 * word, so it must not be called while that stream (or the legacy default
 * stream it may be) is being captured into a CUDA graph.  All calls share
 * the array and each call overwrites it, so calls whose work overlaps on
 * the GPU race: serialise them.  An automatic threshold (thr < 0) is
 * recomputed on every call, since nothing is kept between calls.
 *
 * The column sweep is always the direct kernel (GLSU_METHOD_DIRECT): its
 * output equals glsu_wff_run's bit for bit when that handle also runs the
 * direct kernel, and agrees with the FFT column sweep to FP32 rounding. */
int glsu_wff_run_noalloc(int width, int height, const glsu_wff_params *p, const void *d_f, void *d_filtered,
                         void *cuda_stream);

/* ---- WFR2: WFT2_CUDAF / WFT2_CUDA with WFT_TYPE::WFR -------------------- */
/* WFT/WFT2_CUDAf.h:21-40 (cuWFR2, WFT/WFT2_CUDAf.cu:1174-1319), computed in
 * the formulation of the CPU reference WFT2_cpu::WFR2 (WFT/WFT2_CPU.cpp:
 * 391-694): per pixel the frequency of the largest windowed Fourier
 * coefficient |sf| over the (wx, wy) grid (ties: the later one in wy-major,
 * wx-minor order), its phase, and the curvature least squares.  The eight
 * maps are the WFR fields of WFT2_DeviceResults[F] (WFT/WFT.h:99-135):
 * device arrays of H*W elements of the handle's precision (float or double). */
typedef struct glsu_wfr_results {
    void *wx;          /* local frequency in x of the ridge */
    void *wy;          /* local frequency in y */
    void *phase;       /* angle(sf) at the ridge */
    void *phase_comp;  /* phase compensated by the curvature estimate */
    void *b;           /* amplitude */
    void *r;           /* ridge value max |sf| */
    void *cxx;         /* curvature estimate in x */
    void *cyy;         /* curvature estimate in y */
} glsu_wfr_results;

typedef struct glsu_wfr glsu_wfr;
/* p: sigma, frequency grid (thr is not used); NULL selects the WFR defaults
 * of glsu_wft_default_params(GLSU_WFT_WFR). */
int glsu_wfr_create(glsu_wfr **out, int precision, int width, int height, const glsu_wff_params *p);
int glsu_wfr_destroy(glsu_wfr *h);
int glsu_wfr_set_stream(glsu_wfr *h, void *cuda_stream);
/* WFT2_CUDAF::operator() for WFR: d_f device H*W complex input; the eight
 * device maps of z receive the results; time_ms (may be NULL) the device time. */
int glsu_wfr_run(glsu_wfr *h, const void *d_f, const glsu_wfr_results *z, double *time_ms);
/* Same, enqueued on the handle's stream without waiting. */
int glsu_wfr_run_async(glsu_wfr *h, const void *d_f, const glsu_wfr_results *z);

/* ---- DPRA: DPRA_CUDAF (F32) / DPRA_CUDA (F64) --------------------------- */
/* h_phi0: HOST pointer to W*H initial phase in the handle's precision
 * (copied to the device, as DPRA_CUDAF's constructor does).
 * window_radius r gives a (2r+1)^2 window (the reference hard-wires r=1);
 * wff == NULL selects the reference's hard-wired WFF parameters. */
int glsu_dpra_create(glsu_dpra **out, int precision, const void *h_phi0, int width, int height,
                     int ref_update_rate, int window_radius, const glsu_wff_params *wff);
int glsu_dpra_destroy(glsu_dpra *h);
int glsu_dpra_set_stream(glsu_dpra *h, void *cuda_stream);
/* DPRA_CUDAF::dpra_per_frame: h_img is a HOST frame (img_type GLSU_U8, or
 * the handle's precision), h_dphi receives the HOST W*H phase change.
 * Synchronous; *time_ms (may be NULL) gets the device time including copies. */
int glsu_dpra_per_frame(glsu_dpra *h, const void *h_img, int img_type, void *h_dphi, double *time_ms);
/* Same on device buffers, enqueued on the handle's stream.  d_dphi may be
 * NULL (the phase change stays in the handle). */
int glsu_dpra_per_frame_device(glsu_dpra *h, const void *d_img, int img_type, void *d_dphi);
/* DPRA_CUDAF::update_ref_phi: phi_ref <- phi_curr, dphi_ref <- dphi. */
int glsu_dpra_update_ref_phi(glsu_dpra *h);
/* Batched form (no counterpart in the reference): one frame of each of n
 * independent sequences, handles of any sizes, windows and parameters.
 * d_frames[i] is handle i's device frame (img_type for all), or NULL when
 * its sequence has ended.  Each frame is enqueued on its handle's own stream
 * (so the frames are in flight together; handles in graph mode replay their
 * graphs) and the call returns without waiting.  Each handle follows the
 * sequence rule: after its i-th batched frame the reference is updated when
 * i % rr == 0.  glsu_dpra_batch_wait waits for all of them and reports device
 * errors.  A handle may appear once per step.  On an error at handle i the
 * handles before i have already taken their frame of this step. */
int glsu_dpra_batch_step(glsu_dpra *const *handles, int n, const void *const *d_frames, int img_type);
int glsu_dpra_batch_wait(glsu_dpra *const *handles, int n);
/* Staged batch (no counterpart in the reference): many FP32 plain-form DPRA
 * handles (any sizes, windows and WFF parameters; at most 128 per transform
 * length and launch, more are split) run one frame each per step, stage by
 * stage: per sequence on its own stream the least squares and the WFF2 row
 * pass; then the FFT column sweeps of all sequences that share a transform
 * length as one persistent launch over their (sequence, plane, column group)
 * work list, one launch per length, the lengths on parallel streams
 * (sequences on the direct sweep run it on their own stream); then per
 * sequence the final row pass and the phase update.  Outputs equal each
 * handle's own frames bit for bit.  Each handle follows the sequence rule
 * (after its i-th batched frame the reference is updated when i % rr == 0).
 * glsu_dpra_batch_run returns after enqueueing on the batch's stream;
 * d_frames[i] is handle i's device frame (U8 or F32) or NULL when its
 * sequence has ended.  In graph mode (glsu_dpra_batch_set_graph) each step
 * after the first is one CUDA graph launch (one graph per set of active
 * sequences and reference parities, inputs first copied into the handles'
 * frame buffers).  The handles must outlive the batch and are not used
 * elsewhere while it runs. */
typedef struct glsu_dpra_batch glsu_dpra_batch;
int glsu_dpra_batch_create(glsu_dpra_batch **out, glsu_dpra *const *handles, int n);
int glsu_dpra_batch_destroy(glsu_dpra_batch *b);
int glsu_dpra_batch_set_graph(glsu_dpra_batch *b, int enable);
int glsu_dpra_batch_run(glsu_dpra_batch *b, const void *const *d_frames, int img_type);
/* Waits for the batch's steps and reports device errors. */
int glsu_dpra_batch_sync(glsu_dpra_batch *b);
/* DPRA_CPU::operator() semantics for a block of frames: for frame i, run
 * per_frame, store its dphi, update the reference when i % rr == 0
 * (DPRA/dpra_cpu.cpp:58-89; the CUDA reference's overloads are empty,
 * DPRA/dpra_cudaf.cu:193-205).  h_frames: nframes*W*H host frames;
 * h_dphi_all: nframes*W*H host output.  When both buffers are page-locked
 * (cudaHostAlloc / cudaHostRegister / pinned tensors) the uploads and
 * downloads run on two copy streams of the handle, overlapped with the
 * compute of neighbouring frames, and *time_ms is the device time from the
 * first upload to the last download; otherwise frames go one by one through
 * glsu_dpra_per_frame and *time_ms is the sum of their times.  Results are
 * the same either way.  Returns when every output is on the host. */
int glsu_dpra_sequence(glsu_dpra *h, int nframes, const void *h_frames, int img_type, void *h_dphi_all,
                       double *time_ms);
/* GLSU_LS_FLOAT_FLOAT (default) or GLSU_LS_FP64_SUMS for FP32 handles. */
int glsu_dpra_set_ls_method(glsu_dpra *h, int method);
/* Output tile of the FP32 float-float least squares (the DPRA tile-shape
 * knob): 32 x 16 (the default), 32 x 8 or 32 x 32 outputs per CTA.  The
 * regressors are rotated to each tile's centre phase, so tiles give the
 * same results to float-float rounding, not bit for bit; the default is
 * fixed so that outputs are reproducible unless a tile is chosen.  A tile
 * whose shared memory exceeds the device's per-block limit at the handle's
 * radius (32 x 32 at r = 8) returns GLSU_ERR_UNSUPPORTED. */
int glsu_dpra_set_ls_tile(glsu_dpra *h, int tile_width, int tile_height);
int glsu_dpra_get_ls_tile(const glsu_dpra *h, int *tile_width, int *tile_height);
/* Time the three tiles on this handle's shape and window (a zero frame
 * against its reference phase, three launches each) and select the
 * fastest; ms (optional, 3 floats) receives the times in the order above,
 * -1 for a tile that does not fit at the handle's radius.  Overwrites the handle's frame buffer and least-squares output. */
int glsu_dpra_tune_ls_tile(glsu_dpra *h, float *ms);
/* Copy the last frame's least-squares output exp(j dphi) (complex, W*H) to a
 * device buffer, enqueued on the handle's stream. */
int glsu_dpra_lsq_device(glsu_dpra *h, void *d_out);
/* Copy a state plane (GLSU_PHI_*) to the host. */
int glsu_dpra_get(glsu_dpra *h, int which, void *h_out);
/* Copy exp(j dphi) of the last frame's least-squares stage (W*H complex,
 * the WFF2 input) to the host. */
int glsu_dpra_get_lsq(glsu_dpra *h, void *h_out);
/* Device address of a state plane (valid until the next call on h). */
int glsu_dpra_device_ptr(glsu_dpra *h, int which, void **d_ptr);
/* Spatially unwrap each frame's phase change before adding it to dphi_ref,
 * dphi = dphi_ref + unwrap(t), as MatLab/fp_ls3u.m:104 does; off by default
 * (the C++ reference adds the wrapped t, DPRA/dpra_cpu.cpp:248).  Starts are
 * 0-based; negative selects MATLAB's default (the image centre).  Sides up
 * to 4096. */
int glsu_dpra_set_unwrap(glsu_dpra *h, int enable, int start_row, int start_col);
/* Column-sweep method of the handle's WFF2 (GLSU_METHOD_*). */
int glsu_dpra_set_method(glsu_dpra *h, int method);
/* The handle's column-sweep tuning (see glsu_wff_get_tuning). */
int glsu_dpra_get_tuning(const glsu_dpra *h, glsu_wff_tuning *t);
/* Graph mode (off by default): from the second frame on, the device work of
 * a frame is captured once as a CUDA graph (per input buffer, image type and
 * parity of the exchanged reference buffers) and replayed, which takes the
 * host's per-launch cost out of each frame; device-pointer inputs outside the
 * handle's own buffers are first copied into its frame buffer.  Results are
 * identical to the eager path.  Stage timing runs eagerly. */
int glsu_dpra_set_graph(glsu_dpra *h, int enable);
/* Record CUDA events between the stages of each frame (off by default). */
int glsu_dpra_stage_timing(glsu_dpra *h, int enable);
/* Device times (ms) of the stages of the last frame.  Plain form: [0] LS
 * solve, [1] WFF row pass, [2] WFF column sweep, [3] WFF final row pass +
 * phase update.  Surrogate form: [0] LS solve, [1] network, [2] from the end
 * of the network to the probe residuals (with the probe sweep overlapped:
 * only the part of the sweep the network did not hide), [3] fallback + phase
 * update, then the network split into [4] layer 0, [5] the six tensor-core
 * layers, [6] layer 7, and [7] the probe sweep on its own stream.  Returns the
 * number of stages written (at most n). */
int glsu_dpra_stage_times(glsu_dpra *h, float *ms, int n);

/* ---- spatial unwrapping: MatLab/fp_unwrapping.m ------------------------- */
/* Line-scanning unwrapping of a device H*W phase map (precision GLSU_F32 or
 * GLSU_F64) in place: the column start_col is unwrapped from start_row, then
 * every row from start_col (fp_unwrapping.m:59-71).  0-based starts;
 * negative selects MATLAB's default round(m/2), round(n/2).  Sides up to
 * 4096.  Enqueued on the stream (NULL: legacy default stream). */
int glsu_unwrap2_device(int precision, void *d_p, int width, int height, int start_row, int start_col,
                        void *cuda_stream);

/* ---- AIA: AIA_CUDAF ----------------------------------------------------- */
/* M frames of cols x rows pixels. */
int glsu_aia_create(glsu_aia **out, int M, int cols, int rows);
int glsu_aia_destroy(glsu_aia *h);
int glsu_aia_set_stream(glsu_aia *h, void *cuda_stream);
/* AIA_CUDAF::operator() (AIA/aia_cudaf.cu:308-401).  h_frames: M HOST
 * pointers (img_type GLSU_U8 or GLSU_F32).  h_deltas holds n_deltas_in
 * initial shifts; when n_deltas_in != M they are drawn with
 * glsu_aia_random_deltas(M, seed).  On return h_deltas (M) holds the
 * normalised shifts and h_phi (cols*rows) the wrapped phase. */
int glsu_aia_run(glsu_aia *h, const void *const *h_frames, int img_type, float *h_phi, float *h_deltas,
                 int n_deltas_in, double *time_ms, int *iters, float *err, int max_iter, float max_err,
                 uint64_t seed);
/* Convergence measure of glsu_aia_run: GLSU_AIA_ERR_ABS (the default) is
 * AIA_CUDAF's max_i |delta_i - delta_i,old| (AIA/aia_cpu.cpp:249-263);
 * GLSU_AIA_ERR_RELATIVE is the change of the shifts relative to the first,
 * max_i |(delta_i - delta_0) - (delta_i,old - delta_0,old)|, as
 * AIA_CUDAF_YC2 measures it (AIA/aia_cudaf_v2.cu:665-677).  The phase and
 * frame steps leave a common rotation of all shifts free, and the iterates
 * can drift along it by a constant step per iteration: then the first
 * measure never falls below max_err although the normalised shifts have
 * settled, and the run stops at max_iter. */
#define GLSU_AIA_ERR_ABS 0
#define GLSU_AIA_ERR_RELATIVE 1
int glsu_aia_set_convergence(glsu_aia *h, int mode);
/* Same on M device frames stored back to back (M*cols*rows), enqueued on
 * the stream: the phase stays on the device (d_phi); the deltas (h_deltas,
 * host, in/out as in glsu_aia_run), the iteration count and the error are
 * written after an internal synchronisation. */
int glsu_aia_run_device(glsu_aia *h, const void *d_frames, int img_type, float *d_phi, float *h_deltas,
                        int n_deltas_in, int *iters, float *err, int max_iter, float max_err,
                        uint64_t seed);

/* ---- learned WFF2 surrogate ----------------------------------------------
 * A residual CNN that stands in for WFF2 on DPRA's least-squares output:
 * 8 layers of 3x3 convolutions (per-layer dilations), 32 hidden channels,
 * ReLU; input and output 2 channels (re, im); out = y/|y| with
 * y = z + net(z).  BF16 weights and activations, FP32 accumulation; the
 * 32 -> 32 layers run on the tensor cores (tcgen05).  No reference
 * counterpart: the reference has only the plain WFF2.
 * Parameters (FP32, glsu_sur_param_count() of them): per layer
 * W[co][ci][3][3] then b[co]; layer 0 is 2 -> 32, layers 1..6 32 -> 32,
 * layer 7 32 -> 2.  All device buffers are complex64 [batch][height][width]. */
typedef struct glsu_sur glsu_sur;
int glsu_sur_param_count(void);
/* dilations: 8 values in 1..64.  training != 0 keeps the activations,
 * gradients and Adam state. */
int glsu_sur_create(glsu_sur **out, int batch, int width, int height, const int *dilations, int training);
int glsu_sur_destroy(glsu_sur *h);
int glsu_sur_set_stream(glsu_sur *h, void *cuda_stream);
int glsu_sur_set_params(glsu_sur *h, const float *h_params); /* resets the Adam state */
int glsu_sur_get_params(glsu_sur *h, float *h_params);
/* out = surrogate(d_z), enqueued on the handle's stream. */
int glsu_sur_forward(glsu_sur *h, const void *d_z, void *d_out);
/* Training handles: forward, loss = mean over pixels of
 * min(|t|,1) |out - t/|t||^2 and its gradient for every parameter.  *loss
 * and h_grad (param_count floats) are optional; when given, the call
 * synchronises. */
int glsu_sur_backward(glsu_sur *h, const void *d_z, const void *d_target, double *loss, float *h_grad);
/* Training loss weight of a pixel: min(scale |target|, 1) (scale 1 by
 * default; scale 10 weighs every pixel with |WFF2| >= 0.1 fully, the pixels
 * the probe judges). */
int glsu_sur_set_loss_scale(glsu_sur *h, float scale);
/* One Adam step with the gradient of the last glsu_sur_backward. */
int glsu_sur_adam(glsu_sur *h, float lr, float beta1, float beta2, float eps);
/* Training handles: the output of the last glsu_sur_backward (synchronous). */
int glsu_sur_output(glsu_sur *h, void *h_out);
/* Training crops: for b < batch, copy the width x height window at
 * (row h_crops[3b+1], col h_crops[3b+2]) of pool image h_crops[3b] (pool:
 * complex [pool_n][pool_h][pool_w], input and target) into d_x / d_t.
 * Enqueued on the handle's stream (the crop list is passed by value; at
 * most 512 crops). */
int glsu_sur_gather(glsu_sur *h, const void *d_pool_x, const void *d_pool_t, int pool_n, int pool_h, int pool_w,
                    const int *h_crops, void *d_x, void *d_t);
/* One 32 -> 32 tensor-core layer on caller BF16 NHWC buffers (synchronous):
 * out = relu?(conv_dilation(in, w) + b), zeroed where d_mask <= 0 (d_mask
 * may be NULL).  h_w: W[co][ci][3][3] (rounded to BF16), h_b: [32] or NULL. */
int glsu_sur_conv32(const void *d_in, void *d_out, int batch, int width, int height, int dilation,
                    const float *h_w, const float *h_b, int relu, const void *d_mask, void *cuda_stream);
/* Weight and bias gradient of one 32 -> 32 layer on caller BF16 NHWC buffers
 * (synchronous): d_g the gradient w.r.t. the layer's output, d_in its input;
 * h_dw receives 9216 + 32 floats, dW[co][ci][3][3] then db[co].  The
 * weights on the tensor cores, the bias on CUDA cores, each summed over
 * per-CTA partials in a fixed order. */
int glsu_sur_wgrad32(const void *d_g, const void *d_in, int batch, int width, int height, int dilation,
                     float *h_dw, void *cuda_stream);

/* ---- DPRA surrogate form ---------------------------------------------------
 * FP32 DPRA handles: replace WFF2 by the surrogate (h_params, dilations as
 * above; NULL h_params switches back to the plain WFF2).  Every frame, one
 * patch x patch patch per tile x tile tile gets the exact WFF2 (the sparse
 * probe); tiles whose RMS phase residual exceeds tol (radians) are
 * recomputed by the plain WFF2.  tol <= 0 turns the probes off.  The patch
 * size follows the WFF2 window: 8 for half-sizes round(3 sigma) up to 20, 4
 * from 21 to 45 (patch = 0 selects it; other values are rejected); probes
 * need half-sizes up to 45. */
int glsu_dpra_set_surrogate(glsu_dpra *h, const float *h_params, const int *dilations, int tile, int patch,
                            double tol);
/* Cumulative probe counts; h_resid (optional, one float per tile, tiles
 * row-major) gets the last frame's residuals and h_sites (optional, two ints
 * per tile) the (row, col) of the last frame's probe patches.  Synchronous. */
/* Surrogate form: run the probes' exact WFF2 sweep on a second stream beside
 * the network (enable != 0, the default) with the network's tensor-core
 * layers capped at conv_ctas_per_sm CTAs per SM (0, the default: no cap; 1
 * reserves room on each SM for a probe CTA), or after it on one stream.
 * Measured at 1024^2: 0.580 ms a frame overlapped without a cap, 0.582 with
 * a cap of 2, 0.660 with a cap of 1, 0.613 on one stream. */
int glsu_dpra_set_probe_overlap(glsu_dpra *h, int enable, int conv_ctas_per_sm);
int glsu_dpra_surrogate_stats(glsu_dpra *h, long long *tiles_probed, long long *tiles_flagged, float *h_resid,
                              int *h_sites);

#ifdef __cplusplus
}
#endif

#endif /* GLSU_H */
