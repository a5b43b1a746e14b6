// sur_host.cu -- the surrogate network object: parameters, activation
// buffers, tensor maps, forward / backward / Adam, and its C ABI.  The
// kernels (sur_kernels.cuh) are compiled in this translation unit.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "glsu_internal.cuh"
#include "sur_kernels.cuh"
#include "sur_net.cuh"

namespace glsu {

constexpr int kSurPixBlocks = 152 * 8;  // grid of the per-pixel CUDA-core kernels
constexpr int kSurDbPix = 4096;         // pixels per block of the bias-gradient sums

static int grid_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, kSurPixBlocks); }

// Blocks of the row-walking per-pixel kernels (a block takes whole image rows).
int SurNet::rows_grid() const { return std::min(B * H, kSurPixBlocks); }

int SurNet::last(const float2 *z, float2 *outp, float2 *yp)
{
    SurConvArgs a;
    a.B = B;
    a.H = H;
    a.W = W;
    a.dil = dil[7];
    a.wpack = d_pk7;
    a.bias = d_master + sur_layer_offset(7) + 576;
    a.relu = 0;
    a.err = d_err;
    a.z = z;
    a.cout = outp;
    a.yout = yp;
    a.max_ctas_per_sm = conv_ctas_per_sm;
    return launch_sur_last(map7, a, stream);
}

int SurNet::init(int batch, int width, int height, const int *dilations, bool train)
{
    if (batch < 1 || width < 1 || height < 1) return fail(GLSU_ERR_INVALID, "surrogate: bad batch or size");
    if (!dilations) return fail(GLSU_ERR_INVALID, "surrogate: null dilations");
    for (int l = 0; l < kSurLayers; l++) {
        if (dilations[l] < 1 || dilations[l] > 64) return fail(GLSU_ERR_INVALID, "surrogate: dilation must be 1..64");
        dil[l] = dilations[l];
    }
    B = batch;
    W = width;
    H = height;
    training = train;
    const size_t n = (size_t)B * H * W;
    const size_t abytes = n * 32 * sizeof(uint16_t);
    auto A = [&](void **p, size_t bytes) { return cudaMalloc(p, bytes) == cudaSuccess; };
    bool ok = A((void **)&d_master, kSurParams * 4) && A((void **)&d_pk_fwd, 6 * 9216 * 2) &&
              A((void **)&d_pk_bwd, 6 * 9216 * 2) && A((void **)&d_pk7, kSurPk7Bytes) &&
              A((void **)&d_w0r, 576 * 4) && A((void **)&d_w7r, 576 * 4) &&
              A((void **)&d_err, sizeof(int));
    const int nact = training ? 7 : 2;
    for (int k = 0; k < nact && ok; k++) ok = A((void **)&d_act[k], abytes);
    if (training && ok) {
        ok = A((void **)&d_g[0], abytes) && A((void **)&d_g[1], abytes) && A((void **)&d_dh, n * 8) &&
             A((void **)&d_out, n * 8) && A((void **)&d_grad, kSurParams * 4) && A((void **)&d_m, kSurParams * 4) &&
             A((void **)&d_v, kSurParams * 4) && A((void **)&d_lpart, (size_t)kSurPixBlocks * 8) &&
             A((void **)&d_y, n * 8) &&
             A((void **)&d_loss, 8);
        nbs = sur_dw_small_blocks(B, H, W);
        ndb = (int)((n + kSurDbPix - 1) / kSurDbPix);
        const size_t part = std::max<size_t>(std::max<size_t>((size_t)device_sm_count() * 9216,
                                                              (size_t)nbs * kSurL0Params),
                                             (size_t)ndb * 32);
        ok = ok && A((void **)&d_part, part * 4);
    }
    if (!ok) return fail(GLSU_ERR_ALLOC, "surrogate: device allocation failed");
    GLSU_CUDA_TRY(cudaMemset(d_err, 0, sizeof(int)));
    GLSU_CUDA_TRY(cudaMemset(d_master, 0, kSurParams * 4));
    if (training) {
        GLSU_CUDA_TRY(cudaMemset(d_m, 0, kSurParams * 4));
        GLSU_CUDA_TRY(cudaMemset(d_v, 0, kSurParams * 4));
    }
    // tensor maps: forward layer l reads its input with dilation dil[l]
    for (int l = 1; l <= 6; l++) {
        const void *in = training ? d_act[l - 1] : d_act[(l - 1) & 1];
        const void *out = training ? d_act[l] : d_act[l & 1];
        GLSU_TRY(sur_make_map(&map_fwd[l], in, B, H, W, dil[l]));
        GLSU_TRY(sur_make_out_map(&map_fwd_out[l], out, B, H, W));
        if (training) {
            GLSU_TRY(sur_make_map(&map_bwd[l], d_g[(6 - l) & 1], B, H, W, dil[l]));
            GLSU_TRY(sur_make_out_map(&map_bwd_out[l], d_g[(7 - l) & 1], B, H, W));
        }
    }
    GLSU_TRY(sur_make_map(&map7, a6(), B, H, W, dil[7]));
    if (training)
        for (int k = 0; k < 2; k++) GLSU_TRY(sur_make_map_box(&map_g[k], d_g[k], B, H, W, 128));
    return pack();
}

void SurNet::release()
{
    void *ps[] = {d_master, d_pk_fwd, d_pk_bwd, d_pk7, d_w0r, d_w7r, d_err, d_g[0], d_g[1], d_dh, d_out, d_y,
                  d_grad, d_m, d_v, d_lpart, d_loss, d_part};
    for (void *p : ps) cudaFree(p);
    for (int k = 0; k < 7; k++) cudaFree(d_act[k]);
}

int SurNet::pack()
{
    GLSU_CUDA_TRY(cudaMemsetAsync(d_pk7, 0, kSurPk7Bytes, stream));  // the zero-padded outputs 2..15
    sur_pack_kernel<<<(6 * 9216 + 255) / 256, 256, 0, stream>>>(d_master, d_pk_fwd, d_pk_bwd, d_w0r, d_w7r,
                                                                d_pk7);
    GLSU_CUDA_TRY(cudaGetLastError());
    // layer 0 takes its weights as kernel parameters
    GLSU_CUDA_TRY(cudaMemcpyAsync(h_w0.w, d_w0r, sizeof(h_w0.w), cudaMemcpyDeviceToHost, stream));
    GLSU_CUDA_TRY(cudaMemcpyAsync(h_w0.b, d_master + 576, sizeof(h_w0.b), cudaMemcpyDeviceToHost, stream));
    GLSU_CUDA_TRY(cudaStreamSynchronize(stream));
    return GLSU_OK;
}

int SurNet::set_params(const float *h)
{
    GLSU_CUDA_TRY(cudaMemcpyAsync(d_master, h, kSurParams * 4, cudaMemcpyHostToDevice, stream));
    adam_t = 0;
    if (training) {
        GLSU_CUDA_TRY(cudaMemsetAsync(d_m, 0, kSurParams * 4, stream));
        GLSU_CUDA_TRY(cudaMemsetAsync(d_v, 0, kSurParams * 4, stream));
    }
    GLSU_TRY(pack());
    GLSU_CUDA_TRY(cudaStreamSynchronize(stream));
    return GLSU_OK;
}

int SurNet::get_params(float *h)
{
    GLSU_CUDA_TRY(cudaMemcpyAsync(h, d_master, kSurParams * 4, cudaMemcpyDeviceToHost, stream));
    GLSU_CUDA_TRY(cudaStreamSynchronize(stream));
    return GLSU_OK;
}

int SurNet::check_error()
{
    int e = 0;
    GLSU_CUDA_TRY(cudaMemcpyAsync(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    GLSU_CUDA_TRY(cudaStreamSynchronize(stream));
    if (e) {
        cudaMemsetAsync(d_err, 0, sizeof(int), stream);
        return fail(e, "surrogate kernel: a bounded wait timed out");
    }
    return GLSU_OK;
}

// Layers 0..6: z -> a6 (training: d_act[0..6]; inference: ping-pong).
int SurNet::hidden(const float2 *z, cudaEvent_t *ev)
{
    sur_l0_kernel<<<rows_grid(), 256, 0, stream>>>(z, B, H, W, dil[0], h_w0, d_act[0]);
    GLSU_CUDA_TRY(cudaGetLastError());
    if (ev) GLSU_CUDA_TRY(cudaEventRecord(ev[0], stream));
    for (int l = 1; l <= 6; l++) {
        SurConvArgs a;
        a.B = B;
        a.H = H;
        a.W = W;
        a.dil = dil[l];
        a.wpack = d_pk_fwd + (size_t)(l - 1) * 9216;
        a.bias = d_master + sur_layer_offset(l) + 9216;
        a.mask = nullptr;
        a.out = training ? d_act[l] : d_act[l & 1];
        a.relu = 1;
        a.err = d_err;
        a.max_ctas_per_sm = conv_ctas_per_sm;
        GLSU_TRY(launch_sur_conv(map_fwd[l], map_fwd_out[l], a, stream));
    }
    if (ev) GLSU_CUDA_TRY(cudaEventRecord(ev[1], stream));
    return GLSU_OK;
}

const uint16_t *SurNet::a6() const { return training ? d_act[6] : d_act[0]; }

int SurNet::forward(const void *d_z, void *d_outp, cudaEvent_t *ev)
{
    GLSU_TRY(hidden((const float2 *)d_z, ev));
    return last((const float2 *)d_z, (float2 *)d_outp, nullptr);
}

int SurNet::backward(const void *d_z, const void *d_target)
{
    if (!training) return fail(GLSU_ERR_INVALID, "surrogate handle was not created for training");
    const float2 *z = (const float2 *)d_z;
    GLSU_TRY(hidden(z));
    const int g = rows_grid();
    GLSU_TRY(last(z, nullptr, d_y));
    sur_l7_loss_kernel<<<kSurPixBlocks, 256, 0, stream>>>(d_y, (const float2 *)d_target, (size_t)B * H * W, d_out,
                                                          d_dh, d_lpart, loss_scale);
    sur_sum_kernel<<<1, 32, 0, stream>>>(d_lpart, kSurPixBlocks, d_loss);
    // layer 7: weight gradient and dL/da6 (masked)
    GLSU_TRY(raise_smem_limit((const void *)sur_dw_small_kernel<2, 32>, sur_dw_small_smem(64, 2, 32)));
    GLSU_TRY(raise_smem_limit((const void *)sur_dw_small_kernel<32, 2>, sur_dw_small_smem(64, 32, 2)));
    sur_dw_small_kernel<2, 32><<<nbs, 288, sur_dw_small_smem(dil[7], 2, 32), stream>>>(d_dh, d_act[6], B, H, W,
                                                                                       dil[7], d_part);
    sur_reduce_kernel<<<(kSurL7Params + 31) / 32, sur_reduce_threads(nbs), 0, stream>>>(d_part, nbs, kSurL7Params,
                                                                     d_grad + sur_layer_offset(7));
    sur_l7_bwd_kernel<<<g, 256, 0, stream>>>(d_dh, d_act[6], B, H, W, dil[7], d_w7r, d_g[0]);
    GLSU_CUDA_TRY(cudaGetLastError());
    const size_t npx = (size_t)B * H * W;
    for (int l = 6; l >= 1; l--) {
        uint16_t *gl = d_g[(6 - l) & 1], *gprev = d_g[(7 - l) & 1];
        // weights on the tensor cores, bias on CUDA cores, each summed over its partials in a fixed order
        SurWgradArgs wa;
        wa.B = B;
        wa.H = H;
        wa.W = W;
        wa.dil = dil[l];
        wa.part = d_part;
        wa.err = d_err;
        int nblk = 0;
        GLSU_TRY(launch_sur_wgrad(map_fwd[l], map_g[(6 - l) & 1], wa, stream, &nblk));
        sur_reduce_kernel<<<9216 / 32, sur_reduce_threads(nblk), 0, stream>>>(d_part, nblk, 9216, d_grad + sur_layer_offset(l));
        sur_db32_kernel<<<ndb, 256, 0, stream>>>(gl, npx, kSurDbPix, d_part);
        sur_reduce_kernel<<<1, sur_reduce_threads(ndb), 0, stream>>>(d_part, ndb, 32, d_grad + sur_layer_offset(l) + 9216);
        GLSU_CUDA_TRY(cudaGetLastError());
        SurConvArgs a;
        a.B = B;
        a.H = H;
        a.W = W;
        a.dil = dil[l];
        a.wpack = d_pk_bwd + (size_t)(l - 1) * 9216;
        a.bias = nullptr;
        a.mask = d_act[l - 1];
        a.out = gprev;
        a.relu = 0;
        a.err = d_err;
        GLSU_TRY(launch_sur_conv(map_bwd[l], map_bwd_out[l], a, stream));
    }
    // layer 0: weight gradient from g0 (in d_g[0] after six swaps) and the input
    sur_dw_small_kernel<32, 2><<<nbs, 288, sur_dw_small_smem(dil[0], 32, 2), stream>>>(d_g[0], z, B, H, W, dil[0],
                                                                                       d_part);
    sur_reduce_kernel<<<(kSurL0Params + 31) / 32, sur_reduce_threads(nbs), 0, stream>>>(d_part, nbs, kSurL0Params, d_grad);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

int SurNet::adam(float lr, float b1, float b2, float eps)
{
    if (!training) return fail(GLSU_ERR_INVALID, "surrogate handle was not created for training");
    adam_t++;
    const float c1 = (float)(1.0 / (1.0 - std::pow((double)b1, adam_t)));
    const float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, adam_t)));
    sur_adam_kernel<<<(kSurParams + 255) / 256, 256, 0, stream>>>(d_master, d_grad, d_m, d_v, kSurParams, lr, b1, b2,
                                                                   eps, c1, c2);
    GLSU_CUDA_TRY(cudaGetLastError());
    return pack();
}

}  // namespace glsu

using namespace glsu;

struct glsu_sur {
    SurNet net;
    bool own_stream = false;
};

extern "C" int glsu_sur_param_count(void) { return kSurParams; }

extern "C" int glsu_sur_create(glsu_sur **out, int batch, int width, int height, const int *dilations, int training)
{
    if (!out) return fail(GLSU_ERR_INVALID, "null handle pointer");
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(GLSU_ERR_NO_DEVICE, "no CUDA device visible");
    }
    glsu_sur *h = new glsu_sur();
    int rc = cudaStreamCreateWithFlags(&h->net.stream, cudaStreamNonBlocking) == cudaSuccess
                 ? GLSU_OK
                 : fail(GLSU_ERR_CUDA, "cudaStreamCreate failed");
    h->own_stream = rc == GLSU_OK;
    if (rc == GLSU_OK) rc = h->net.init(batch, width, height, dilations, training != 0);
    if (rc == GLSU_OK) rc = cudaStreamSynchronize(h->net.stream) == cudaSuccess ? GLSU_OK : GLSU_ERR_CUDA;
    if (rc != GLSU_OK) {
        glsu_sur_destroy(h);
        return rc;
    }
    *out = h;
    return GLSU_OK;
}

extern "C" int glsu_sur_destroy(glsu_sur *h)
{
    if (!h) return GLSU_OK;
    if (h->net.stream) cudaStreamSynchronize(h->net.stream);
    h->net.release();
    if (h->own_stream && h->net.stream) cudaStreamDestroy(h->net.stream);
    delete h;
    return GLSU_OK;
}

extern "C" int glsu_sur_set_stream(glsu_sur *h, void *stream)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    if (h->own_stream && h->net.stream) {
        cudaStreamSynchronize(h->net.stream);
        cudaStreamDestroy(h->net.stream);
    }
    h->net.stream = (cudaStream_t)stream;
    h->own_stream = false;
    return GLSU_OK;
}

extern "C" int glsu_sur_set_params(glsu_sur *h, const float *params)
{
    if (!h || !params) return fail(GLSU_ERR_INVALID, "null argument");
    return h->net.set_params(params);
}

extern "C" int glsu_sur_get_params(glsu_sur *h, float *params)
{
    if (!h || !params) return fail(GLSU_ERR_INVALID, "null argument");
    return h->net.get_params(params);
}

extern "C" int glsu_sur_forward(glsu_sur *h, const void *d_z, void *d_out)
{
    if (!h || !d_z || !d_out) return fail(GLSU_ERR_INVALID, "null argument");
    return h->net.forward(d_z, d_out);
}

extern "C" int glsu_sur_backward(glsu_sur *h, const void *d_z, const void *d_target, double *loss, float *h_grad)
{
    if (!h || !d_z || !d_target) return fail(GLSU_ERR_INVALID, "null argument");
    GLSU_TRY(h->net.backward(d_z, d_target));
    if (loss || h_grad) {
        if (loss) GLSU_CUDA_TRY(cudaMemcpyAsync(loss, h->net.d_loss, 8, cudaMemcpyDeviceToHost, h->net.stream));
        if (h_grad)
            GLSU_CUDA_TRY(
                cudaMemcpyAsync(h_grad, h->net.d_grad, kSurParams * 4, cudaMemcpyDeviceToHost, h->net.stream));
        GLSU_TRY(h->net.check_error());
    }
    return GLSU_OK;
}

extern "C" int glsu_sur_set_loss_scale(glsu_sur *h, float scale)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    if (!(scale > 0.f) || !std::isfinite(scale)) return fail(GLSU_ERR_INVALID, "loss scale must be positive");
    h->net.loss_scale = scale;
    return GLSU_OK;
}

extern "C" int glsu_sur_adam(glsu_sur *h, float lr, float beta1, float beta2, float eps)
{
    if (!h) return fail(GLSU_ERR_INVALID, "null handle");
    return h->net.adam(lr, beta1, beta2, eps);
}

extern "C" int glsu_sur_output(glsu_sur *h, void *h_out)
{
    if (!h || !h_out) return fail(GLSU_ERR_INVALID, "null argument");
    if (!h->net.training) return fail(GLSU_ERR_INVALID, "only training handles keep their last output");
    const size_t n = (size_t)h->net.B * h->net.H * h->net.W;
    GLSU_CUDA_TRY(cudaMemcpyAsync(h_out, h->net.d_out, n * 8, cudaMemcpyDeviceToHost, h->net.stream));
    return h->net.check_error();
}

extern "C" int glsu_sur_gather(glsu_sur *h, const void *d_pool_x, const void *d_pool_t, int pool_n, int pool_h,
                               int pool_w, const int *h_crops, void *d_x, void *d_t)
{
    if (!h || !d_pool_x || !d_pool_t || !h_crops || !d_x || !d_t) return fail(GLSU_ERR_INVALID, "null argument");
    SurNet &N = h->net;
    if (N.B > kSurMaxBatch) return fail(GLSU_ERR_UNSUPPORTED, "gather: at most 512 crops a batch");
    SurCrops c;
    for (int b = 0; b < N.B; b++) {
        const int oy = h_crops[3 * b + 1], ox = h_crops[3 * b + 2];
        if (h_crops[3 * b] < 0 || h_crops[3 * b] >= pool_n || oy < 0 || ox < 0 || oy + N.H > pool_h ||
            ox + N.W > pool_w)
            return fail(GLSU_ERR_INVALID, "crop outside the pool image");
        c.c[b] = make_int4(h_crops[3 * b], oy, ox, 0);
    }
    const size_t n = (size_t)N.B * N.H * N.W;
    sur_gather_kernel<<<grid_for(n), 256, 0, N.stream>>>((const float2 *)d_pool_x, (const float2 *)d_pool_t, pool_h,
                                                         pool_w, c, N.B, N.H, N.W, (float2 *)d_x, (float2 *)d_t);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

// One 32 -> 32 tensor-core convolution on caller buffers (the building block
// of the hidden layers; synchronous).  w: W[co][ci][3][3] FP32 (rounded to
// BF16 here), b: [32] or NULL.
extern "C" int glsu_sur_conv32(const void *d_in, void *d_out, int batch, int width, int height, int dilation,
                               const float *h_w, const float *h_b, int relu, const void *d_mask, void *stream)
{
    if (!d_in || !d_out || !h_w) return fail(GLSU_ERR_INVALID, "null argument");
    if (batch < 1 || width < 1 || height < 1) return fail(GLSU_ERR_INVALID, "bad size");
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<float> master(kSurParams, 0.f);
    std::memcpy(master.data() + sur_layer_offset(1), h_w, 9216 * 4);
    if (h_b) std::memcpy(master.data() + sur_layer_offset(1) + 9216, h_b, 32 * 4);
    float *d_master = nullptr, *d_w0r = nullptr, *d_w7r = nullptr;
    uint16_t *d_pk = nullptr, *d_pkb = nullptr;
    int *d_err = nullptr;
    int rc = GLSU_OK;
    if (cudaMalloc(&d_master, kSurParams * 4) != cudaSuccess || cudaMalloc(&d_pk, 6 * 9216 * 2) != cudaSuccess ||
        cudaMalloc(&d_pkb, 6 * 9216 * 2) != cudaSuccess || cudaMalloc(&d_w0r, 576 * 4) != cudaSuccess ||
        cudaMalloc(&d_w7r, 576 * 4) != cudaSuccess || cudaMalloc(&d_err, 4) != cudaSuccess)
        rc = fail(GLSU_ERR_ALLOC, "allocation failed");
    CUtensorMap tm, tmo;
    if (rc == GLSU_OK) rc = sur_make_map(&tm, d_in, batch, height, width, dilation);
    if (rc == GLSU_OK) rc = sur_make_out_map(&tmo, d_out, batch, height, width);
    if (rc == GLSU_OK) {
        cudaMemcpyAsync(d_master, master.data(), kSurParams * 4, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(d_err, 0, 4, s);
        sur_pack_kernel<<<(6 * 9216 + 255) / 256, 256, 0, s>>>(d_master, d_pk, d_pkb, d_w0r, d_w7r, nullptr);
        SurConvArgs a;
        a.B = batch;
        a.H = height;
        a.W = width;
        a.dil = dilation;
        a.wpack = d_pk;
        a.bias = h_b ? d_master + sur_layer_offset(1) + 9216 : nullptr;
        a.mask = (const uint16_t *)d_mask;
        a.out = (uint16_t *)d_out;
        a.relu = relu;
        a.err = d_err;
        rc = launch_sur_conv(tm, tmo, a, s);
    }
    int e = 0;
    if (rc == GLSU_OK && cudaMemcpyAsync(&e, d_err, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        rc = fail(GLSU_ERR_CUDA, "copy failed");
    if (rc == GLSU_OK && cudaStreamSynchronize(s) != cudaSuccess) rc = fail(GLSU_ERR_CUDA, "conv failed");
    if (rc == GLSU_OK && e) rc = fail(e, "conv: a bounded wait timed out");
    cudaFree(d_master);
    cudaFree(d_pk);
    cudaFree(d_pkb);
    cudaFree(d_w0r);
    cudaFree(d_w7r);
    cudaFree(d_err);
    return rc;
}

namespace glsu {
int sur_wgrad32_once(const void *d_g, const void *d_in, int batch, int width, int height, int dilation, float *h_dw,
                     cudaStream_t s)
{
    const size_t n = (size_t)batch * height * width;
    const int ndb = (int)((n + kSurDbPix - 1) / kSurDbPix);
    float *d_part = nullptr, *d_out = nullptr;
    int *d_err = nullptr;
    int rc = GLSU_OK;
    const size_t part = std::max<size_t>((size_t)device_sm_count() * 9216, (size_t)ndb * 32);
    if (cudaMalloc(&d_part, part * 4) != cudaSuccess || cudaMalloc(&d_out, kSurL32Params * 4) != cudaSuccess ||
        cudaMalloc(&d_err, 4) != cudaSuccess)
        rc = fail(GLSU_ERR_ALLOC, "allocation failed");
    CUtensorMap tma, tmg;
    if (rc == GLSU_OK) rc = sur_make_map(&tma, d_in, batch, height, width, dilation);
    if (rc == GLSU_OK) rc = sur_make_map_box(&tmg, d_g, batch, height, width, 128);
    if (rc == GLSU_OK && cudaMemsetAsync(d_err, 0, 4, s) != cudaSuccess) rc = fail(GLSU_ERR_CUDA, "memset failed");
    if (rc == GLSU_OK) {
        SurWgradArgs wa;
        wa.B = batch;
        wa.H = height;
        wa.W = width;
        wa.dil = dilation;
        wa.part = d_part;
        wa.err = d_err;
        int nblk = 0;
        rc = launch_sur_wgrad(tma, tmg, wa, s, &nblk);
        if (rc == GLSU_OK) {
            sur_reduce_kernel<<<9216 / 32, sur_reduce_threads(nblk), 0, s>>>(d_part, nblk, 9216, d_out);
            sur_db32_kernel<<<ndb, 256, 0, s>>>((const uint16_t *)d_g, n, kSurDbPix, d_part);
            sur_reduce_kernel<<<1, sur_reduce_threads(ndb), 0, s>>>(d_part, ndb, 32, d_out + 9216);
            if (cudaGetLastError() != cudaSuccess) rc = fail(GLSU_ERR_CUDA, "weight-gradient launch failed");
        }
    }
    int e = 0;
    if (rc == GLSU_OK && (cudaMemcpyAsync(h_dw, d_out, kSurL32Params * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                          cudaMemcpyAsync(&e, d_err, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess))
        rc = fail(GLSU_ERR_CUDA, "copy failed");
    if (rc == GLSU_OK && cudaStreamSynchronize(s) != cudaSuccess) rc = fail(GLSU_ERR_CUDA, "weight gradient failed");
    if (rc == GLSU_OK && e) rc = fail(e, "weight gradient: a bounded wait timed out");
    cudaFree(d_part);
    cudaFree(d_out);
    cudaFree(d_err);
    return rc;
}
}  // namespace glsu

// Weight and bias gradient of one 32 -> 32 layer on caller buffers (the
// building block of the training pass; synchronous).  d_g: the gradient
// w.r.t. the layer's output, d_in: its input, both [B][H][W][32] BF16;
// h_dw: 9216 + 32 floats, W[co][ci][3][3] then b[co].
extern "C" int glsu_sur_wgrad32(const void *d_g, const void *d_in, int batch, int width, int height, int dilation,
                                float *h_dw, void *stream)
{
    if (!d_g || !d_in || !h_dw) return glsu::fail(GLSU_ERR_INVALID, "null argument");
    if (batch < 1 || width < 1 || height < 1) return glsu::fail(GLSU_ERR_INVALID, "bad size");
    return glsu::sur_wgrad32_once(d_g, d_in, batch, width, height, dilation, h_dw, (cudaStream_t)stream);
}
