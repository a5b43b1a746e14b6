// sur_net.cuh -- the surrogate network object shared by the C ABI and the
// DPRA handle (see sur_kernels.cuh for the network and its kernels).
#pragma once

#include "glsu_internal.cuh"

namespace glsu {

struct SurNet {
    int B = 0, H = 0, W = 0;
    int dil[kSurLayers] = {1, 1, 1, 1, 1, 1, 1, 1};
    bool training = false;
    cudaStream_t stream = nullptr;
    // parameters: FP32 master, BF16 operand images of layers 1..6 (forward and
    // transposed/flipped for backward-data) and of layer 7, BF16-rounded
    // layers 0 and 7
    float *d_master = nullptr;
    uint16_t *d_pk_fwd = nullptr, *d_pk_bwd = nullptr, *d_pk7 = nullptr;
    float *d_w0r = nullptr, *d_w7r = nullptr;
    SurL0W h_w0;  // host copy of layer 0 (kernel-parameter weights)
    // activations [B][H][W][32] BF16: training keeps a0..a6, inference ping-pongs two
    uint16_t *d_act[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // training
    uint16_t *d_g[2] = {nullptr, nullptr};  // gradients w.r.t. pre-activations
    float2 *d_dh = nullptr, *d_out = nullptr, *d_y = nullptr;  // y = z + h7 before the renormalisation
    float *d_grad = nullptr, *d_m = nullptr, *d_v = nullptr, *d_part = nullptr;
    double *d_lpart = nullptr, *d_loss = nullptr;
    int nbs = 0, ndb = 0, adam_t = 0;  // blocks of the small weight-gradient and bias-gradient kernels
    int conv_ctas_per_sm = 0;  // cap of the tensor-core layers' CTAs per SM (0: none)
    float loss_scale = 1.f;    // training loss weight min(loss_scale |target|, 1)
    int *d_err = nullptr;
    CUtensorMap map_fwd[7], map_bwd[7];        // conv inputs (box 128 + 2d)
    CUtensorMap map_fwd_out[7], map_bwd_out[7];  // conv outputs (32-pixel tiles)
    CUtensorMap map7;                            // the last layer's input a6
    CUtensorMap map_g[2];                        // d_g[0], d_g[1] in 128-pixel boxes (weight gradients)

    int init(int batch, int width, int height, const int *dilations, bool train);
    void release();
    int pack();
    int set_params(const float *h);
    int get_params(float *h);
    // layers 0..6; ev (optional, 2 events) is recorded after layer 0 and after layer 6
    int hidden(const float2 *z, cudaEvent_t *ev = nullptr);
    const uint16_t *a6() const;
    // out = y / |y| of the network on z (complex [B][H][W]), enqueued on stream
    int forward(const void *d_z, void *d_out, cudaEvent_t *ev = nullptr);
    // forward with loss and all parameter gradients into d_grad / d_loss
    int backward(const void *d_z, const void *d_target);
    int adam(float lr, float b1, float b2, float eps);
    int check_error();
    int rows_grid() const;
    // the last layer on the tensor cores: out = y/|y| into outp, or y into yp
    int last(const float2 *z, float2 *outp, float2 *yp);
};

}  // namespace glsu
