// sur_kernels.cuh -- kernels of the learned WFF2 surrogate on sm_103a
// (compiled in sur_host.cu).
//
// Network: 8 layers of 3x3 convolutions with per-layer dilation, 32 hidden
// channels, ReLU after layers 0..6; input and output 2 channels (re, im):
//     x   = (Re z, Im z)                 z = exp(j dphi) of the DPRA LS stage
//     a0  = relu(conv0(x))               2 -> 32   CUDA cores, FP32 math
//     a_l = relu(conv_l(a_{l-1}))        32 -> 32  tcgen05, l = 1..6
//     y   = x + conv7(a6)                32 -> 2   CUDA cores
//     out = y / |y|                      the stand-in for WFF2(z) / |WFF2(z)|
// Weights and activations are BF16, accumulation FP32 (TMEM for the
// tensor-core layers).  Activations are NHWC [B][H][W][32] BF16, 64 bytes a
// pixel.
//
// Tensor-core layer (sur_conv_tc_kernel): the MMA tile is 128 consecutive
// pixels of one row (M = 128), K = 16 input channels per tcgen05.mma.  The
// input rows are loaded by TMA through a 4-D tensor map {32 channels, W, H,
// B} with box {32, 128 + 2d, 1, 1} and 64-byte swizzle: each pixel's 64
// bytes arrive as one line, and in shared memory they form the K-major
// SWIZZLE_64B operand layout (rows of 64 bytes, 8-row groups 512 bytes
// apart, the 16-byte chunks of a row permuted by address bits 7-8).  A tap's
// horizontal offset dx * d is a shift of the descriptor start by 64 * dx * d
// bytes, the second K = 16 half a shift by 32 bytes, with the base offset
// field left at 0: the tensor core applies the swizzle to the absolute
// shared-memory address, as TMA does (measured: every dilation 1..16 and odd
// shifts agree with the oracle), so no im2col copy is needed, and TMA
// zero-fills the image border.  The epilogue writes each warp's 32 output pixels into a
// staging tile in the same swizzled layout (conflict-free 16-byte stores)
// and one thread stores the tile with a TMA tensor store.
// Work items are chunks of kSurRows output rows of one chain y = r, r + d,
// r + 2d, ... (the rows that share input rows under dilation d).  Input row j
// of an item (j = 0 .. nout + 1) feeds output rows j - 2, j - 1, j through
// the vertical taps dy = 2, 1, 0, so each input row is consumed by ONE MMA
// per (dx, K half) with N = 96: the B operand stacks the three vertical taps'
// weights [dy = 2 | dy = 1 | dy = 0] and the D columns are the three output
// rows' accumulators, which sit side by side in TMEM (output row k of the
// item at columns 32k .. 32k + 31).  At the ends of an item N shrinks to 64
// or 32.  Every MMA accumulates: the epilogue fills each accumulator with the
// bias before its first use and again after draining it.  A row's 18 K = 16
// products are thus 6 MMAs of up to N = 96 instead of 18 of N = 32 (an N = 32
// MMA costs nearly as much as an N = 96 one).
// The kernel is persistent and warp-specialised: one thread streams every
// item's input rows through a ring of slots by TMA, one thread issues the
// MMAs, four warps drain the accumulators.
#pragma once

#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cmath>

#include "glsu_internal.cuh"
#include "ptx_sm103.cuh"

namespace glsu {

constexpr int kSurSlots = 8;     // input-row ring of the tensor-core conv (TMA loads in flight)
constexpr int kSurRows = 8;      // output rows per work item = TMEM accumulators
constexpr int kSurWBytes = 9 * 4 * 32 * 16;  // packed B operand of a 32 -> 32 layer
constexpr int kSurStageBytes = 32 * 64;      // one epilogue warp's output tile

// Geometry of a tensor-core layer with NOUT output channels per accumulator:
// 32 for the hidden layers, 16 for the last layer (its 2 outputs padded with
// zero weights to the smallest N of an M = 128 MMA).  The packed B operand
// is [dx][K half kc][8-channel chunk h][3 NOUT rows][8 channels], row
// n = NOUT (2 - dy) + output channel.
template <int NOUT> struct SurTc {
    static constexpr int BROWS = 3 * NOUT;
    static constexpr int BHALF = BROWS * 16;  // bytes between the two 8-channel chunks of one K = 16 step
    static constexpr int BSTEP = 2 * BHALF;   // bytes of one (dx, kc) operand
    static constexpr int WBYTES = 6 * BSTEP;  // 3 dx x 2 kc operands (a 1024-byte multiple)
    static constexpr int TMEM_COLS = kSurRows * NOUT;
    static constexpr int STAGE = NOUT == 32 ? 4 * kSurStageBytes : 0;
    static constexpr int NBIAS = NOUT == 32 ? 32 : 2;
};
static_assert(SurTc<32>::WBYTES == kSurWBytes && SurTc<16>::WBYTES % 1024 == 0, "B operand layout");
constexpr int kSurPk7Bytes = SurTc<16>::WBYTES;  // packed B operand of the last layer

// out = y / |y| with the same rounding wherever it is evaluated (the last
// layer's epilogue in inference, the loss kernel in training).
__device__ __forceinline__ void sur_unit(float yr, float yi, float &orr, float &oii, float &inv)
{
    const float nrm = __fsqrt_rn(__fadd_rn(__fmul_rn(yr, yr), __fmul_rn(yi, yi)));
    inv = nrm > 1e-20f ? __fdiv_rn(1.f, nrm) : 0.f;
    orr = __fmul_rn(yr, inv);
    oii = __fmul_rn(yi, inv);
}

__device__ __forceinline__ float bf2f(uint16_t v) { return __uint_as_float((uint32_t)v << 16); }

__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&h);
}

__device__ __forceinline__ void unpack8(const uint4 u, float *f)
{
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        f[2 * i] = __uint_as_float(w[i] << 16);
        f[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
    }
}

// ---------------------------------------------------------------------------
// tensor-core 32 -> 32 conv (forward, or backward-data with flipped weights)
// ---------------------------------------------------------------------------
// Work item: (image b, 128-pixel segment, residue r mod d, chunk of the
// chain r, r+d, r+2d, ...), up to kSurRows output rows with 2 halo rows.
struct SurItem {
    int b, x0, r, kbeg, nout;
};

__device__ __forceinline__ SurItem sur_item(const SurConvArgs &a, int item)
{
    const int nsx = (a.W + 127) / 128;
    const int nch = ((a.H + a.dil - 1) / a.dil + kSurRows - 1) / kSurRows;
    SurItem it;
    const int ch = item % nch;
    item /= nch;
    it.r = item % a.dil;
    item /= a.dil;
    it.x0 = (item % nsx) * 128;
    it.b = item / nsx;
    it.kbeg = ch * kSurRows;
    const int chain_len = (a.H - it.r + a.dil - 1) / a.dil;  // rows r, r+d, ... below H
    it.nout = max(0, min(kSurRows, chain_len - it.kbeg));
    return it;
}

// Persistent, warp-specialised: thread 0 of warp 0 issues the TMA row loads
// into a ring of kSurSlots slots, thread 0 of warp 1 issues the MMAs, warps
// 4-7 drain the accumulators.  All three walk the same item list
// (blockIdx.x, + gridDim.x, ...); input rows are numbered across items and
// each accumulator completes one phase of its two mbarriers per item (a
// block that an item leaves unused gets an empty phase), which keeps the
// mbarrier parities consistent.  NOUT = 32: a hidden layer (ReLU / mask,
// BF16 NHWC by TMA store through tmo); NOUT = 16: the last layer (y = z +
// conv + bias from the first two accumulator columns; out = y / |y| into
// a.cout, or y itself into a.yout).
template <int NOUT>
__global__ void __launch_bounds__(256, 1) sur_conv_tc_kernel(const __grid_constant__ CUtensorMap tm,
                                                             const __grid_constant__ CUtensorMap tmo, SurConvArgs a,
                                                             int nitems)
{
    using L = SurTc<NOUT>;
    extern __shared__ __align__(1024) unsigned char sm[];
    const int BW = 128 + 2 * a.dil;
    const int slot_bytes = (BW * 64 + 1023) & ~1023;
    unsigned char *wsm = sm;
    unsigned char *slots = sm + L::WBYTES;
    unsigned char *stage = slots + kSurSlots * slot_bytes;  // [4 warps][32 px][64 B], 64-byte swizzle
    uint64_t *full = reinterpret_cast<uint64_t *>(stage + L::STAGE);
    uint64_t *sfree = full + kSurSlots;
    uint64_t *accf = sfree + kSurSlots;  // [kSurRows] accumulator complete
    uint64_t *acce = accf + kSurRows;    // [kSurRows] accumulator drained and refilled with the bias
    uint64_t *drain = acce + kSurRows;
    float *bias_s = reinterpret_cast<float *>(drain + 1);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bias_s + 32);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < kSurSlots; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&sfree[s], 1);
        }
        for (int b = 0; b < kSurRows; b++) {
            mbar_init(&accf[b], 1);
            mbar_init(&acce[b], 128);
        }
        mbar_init(drain, 1);
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(tslot, L::TMEM_COLS);
    for (int e = tid; e < L::WBYTES / 16; e += 256)
        reinterpret_cast<uint4 *>(wsm)[e] = reinterpret_cast<const uint4 *>(a.wpack)[e];
    if (tid < 32) bias_s[tid] = (a.bias && tid < L::NBIAS) ? a.bias[tid] : 0.f;
    fence_proxy_async_smem();  // the weight image was written by generic stores
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0 && lane == 0) {
        // ---- producer: TMA loads of every item's nout + 2 input rows ----
        uint32_t g = 0;
        bool ok = true;
        for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
            const SurItem it = sur_item(a, item);
            for (int j = 0; j < it.nout + 2 && it.nout > 0; j++, g++) {
                const int s = g % kSurSlots;
                if (g >= kSurSlots && !mbar_wait_bounded(&sfree[s], ((g / kSurSlots) - 1) & 1)) {
                    ok = false;
                    break;
                }
                mbar_expect_tx(&full[s], (uint32_t)BW * 64);
                tma_load_4d(slots + s * slot_bytes, &tm, &full[s], 0, it.x0 - a.dil, it.r + (it.kbeg + j - 1) * a.dil,
                            it.b);
            }
        }
        if (!ok) atomicExch(a.err, GLSU_ERR_TIMEOUT);
        // every load has landed before the CTA exits
        for (uint32_t j = g > (uint32_t)kSurSlots ? g - kSurSlots : 0; j < g; j++)
            mbar_wait_bounded(&full[j % kSurSlots], (j / kSurSlots) & 1);
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        const uint32_t wbase = smem_u32(wsm), sbase = smem_u32(slots);
        uint32_t g = 0, li = 0;
        bool ok = true;
        for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x, li++) {
            const SurItem it = sur_item(a, item);
            if (it.nout <= 0) {
                li--;
                continue;
            }
            const uint32_t par = li & 1;
            for (int j = 0; j < it.nout + 2 && ok; j++, g++) {
                const int s = g % kSurSlots;
                if (!mbar_wait_bounded(&full[s], (g / kSurSlots) & 1)) ok = false;
                // output row j is first written by this input row: its accumulator must hold the bias
                if (ok && j < it.nout && !mbar_wait_bounded(&acce[j], par)) ok = false;
                if (!ok) break;
                tc_fence_after();
                const int klo = max(0, j - 2), khi = min(it.nout - 1, j);
                const uint32_t id = khi == klo       ? umma_idesc_bf16(128, NOUT)
                                    : khi == klo + 1 ? umma_idesc_bf16(128, 2 * NOUT)
                                                     : umma_idesc_bf16(128, 3 * NOUT);
                const uint32_t d = tmem + (uint32_t)(klo * NOUT);
                const uint32_t srow = sbase + (uint32_t)(s * slot_bytes);
                const uint32_t brow = wbase + (uint32_t)((2 - j + klo) * NOUT * 16);
#pragma unroll
                for (int dx = 0; dx < 3; dx++) {
#pragma unroll
                    for (int kc = 0; kc < 2; kc++) {
                        const uint32_t astart = srow + (uint32_t)(dx * a.dil * 64 + kc * 32);
                        const uint64_t ad = umma_desc_sw64(astart, 0);
                        const uint64_t bd = umma_desc(brow + (uint32_t)((dx * 2 + kc) * L::BSTEP), L::BHALF, 128);
                        umma_bf16(d, ad, bd, id, 1u);
                    }
                }
                umma_commit(&sfree[s]);              // input row g is not read again
                if (j >= 2) umma_commit(&accf[j - 2]);  // output row j - 2 has all its products
            }
            // accumulators this item leaves unused: an empty phase
            for (int b = it.nout; b < kSurRows && ok; b++) {
                if (!mbar_wait_bounded(&acce[b], par)) ok = false;
                else umma_commit(&accf[b]);
            }
        }
        if (!ok) atomicExch(a.err, GLSU_ERR_TIMEOUT);
        umma_commit(drain);  // every MMA has completed before TMEM is released
        mbar_wait_bounded(drain, 0);
    } else if (warp >= 4 && NOUT == 16) {
        // ---- last-layer epilogue: y = z + h, out = y / |y|; refill with the bias ----
        const int q = warp - 4;
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
        float bias[16];
#pragma unroll
        for (int c = 0; c < 16; c++) bias[c] = bias_s[c];
        for (int b = 0; b < kSurRows; b++) tmem_st16(lane_base + b * NOUT, bias);
        tc_fence_before();
        for (int b = 0; b < kSurRows; b++) mbar_arrive(&acce[b]);
        uint32_t li = 0;
        bool ok = true;
        for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
            const SurItem it = sur_item(a, item);
            if (it.nout <= 0) continue;
            const int x = it.x0 + q * 32 + lane;
            // the residual input z of the item's rows, loaded before the first
            // accumulator wait so that the loads overlap the MMAs
            float2 zr[kSurRows];
#pragma unroll
            for (int k = 0; k < kSurRows; k++) {
                zr[k] = make_float2(0.f, 0.f);
                if (k < it.nout && x < a.W)
                    zr[k] = a.z[((size_t)it.b * a.H + it.r + (size_t)(it.kbeg + k) * a.dil) * a.W + x];
            }
#pragma unroll
            for (int k = 0; k < kSurRows; k++) {
                if (!__all_sync(0xffffffffu, mbar_wait_bounded(&accf[k], li & 1))) {
                    if (lane == 0) atomicExch(a.err, GLSU_ERR_TIMEOUT);
                    ok = false;
                    break;
                }
                tc_fence_after();
                float h[2] = {0.f, 0.f};
                if (k < it.nout) {
                    tmem_ld2(lane_base + k * NOUT, h);
                    tmem_st16(lane_base + k * NOUT, bias);
                }
                tc_fence_before();
                mbar_arrive(&acce[k]);
                if (k >= it.nout || x >= a.W) continue;
                const size_t p = ((size_t)it.b * a.H + it.r + (size_t)(it.kbeg + k) * a.dil) * a.W + x;
                const float2 zv = zr[k];
                const float yr = __fadd_rn(zv.x, h[0]), yi = __fadd_rn(zv.y, h[1]);
                if (a.yout) {
                    a.yout[p] = make_float2(yr, yi);
                } else {
                    float orr, oii, inv;
                    sur_unit(yr, yi, orr, oii, inv);
                    a.cout[p] = make_float2(orr, oii);
                }
            }
            li++;
        }
    } else if (warp >= 4 && NOUT == 32) {
        // ---- epilogue: TMEM -> ReLU, mask -> BF16 NHWC; refill with the bias ----
        const int q = warp - 4;
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
        unsigned char *my_stage = stage + q * kSurStageBytes;
        float bias[32];
#pragma unroll
        for (int c = 0; c < 32; c++) bias[c] = bias_s[c];
        for (int b = 0; b < kSurRows; b++) tmem_st32(lane_base + b * 32, bias);
        tc_fence_before();
        for (int b = 0; b < kSurRows; b++) mbar_arrive(&acce[b]);
        uint32_t li = 0;
        bool ok = true;
        for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
            const SurItem it = sur_item(a, item);
            if (it.nout <= 0) continue;
            const int x = it.x0 + q * 32 + lane;
            for (int k = 0; k < kSurRows; k++) {
                // warp-uniform: tcgen05.ld / st below are warp-collective instructions
                if (!__all_sync(0xffffffffu, mbar_wait_bounded(&accf[k], li & 1))) {
                    if (lane == 0) atomicExch(a.err, GLSU_ERR_TIMEOUT);
                    ok = false;
                    break;
                }
                tc_fence_after();
                float v[32];
                if (k < it.nout) {
                    tmem_ld32(lane_base + k * 32, v);
                    tmem_st32(lane_base + k * 32, bias);
                }
                tc_fence_before();
                mbar_arrive(&acce[k]);
                if (k >= it.nout) continue;
                const int y = it.r + (it.kbeg + k) * a.dil;
                if (a.relu) {
#pragma unroll
                    for (int c = 0; c < 32; c++) v[c] = fmaxf(v[c], 0.f);
                }
                if (a.mask && x < a.W) {
                    const uint4 *mp =
                        reinterpret_cast<const uint4 *>(a.mask + (((size_t)it.b * a.H + y) * a.W + x) * 32);
#pragma unroll
                    for (int g = 0; g < 4; g++) {
                        float mv[8];
                        unpack8(mp[g], mv);
#pragma unroll
                        for (int i = 0; i < 8; i++)
                            if (!(mv[i] > 0.f)) v[8 * g + i] = 0.f;
                    }
                }
                // the previous tile of this warp has been read by its TMA store
                if (lane == 0) bulk_wait_read0();
                __syncwarp();
#pragma unroll
                for (int g = 0; g < 4; g++)
                    *reinterpret_cast<uint4 *>(my_stage + lane * 64 + ((g ^ ((lane >> 1) & 3)) * 16)) =
                        make_uint4(pack_bf2(v[8 * g], v[8 * g + 1]), pack_bf2(v[8 * g + 2], v[8 * g + 3]),
                                   pack_bf2(v[8 * g + 4], v[8 * g + 5]), pack_bf2(v[8 * g + 6], v[8 * g + 7]));
                fence_proxy_async_smem();
                __syncwarp();
                // columns beyond W are clipped by the store
                if (lane == 0 && it.x0 + q * 32 < a.W) {
                    tma_store_4d(&tmo, my_stage, 0, it.x0 + q * 32, y, it.b);
                    bulk_commit();
                }
            }
            li++;
        }
        if (lane == 0) bulk_wait0();  // every output tile has been written
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, L::TMEM_COLS);
}

template <int NOUT> static int sur_conv_smem_bytes(int dil)
{
    const int BW = 128 + 2 * dil;
    const int slot_bytes = (BW * 64 + 1023) & ~1023;
    return SurTc<NOUT>::WBYTES + kSurSlots * slot_bytes + SurTc<NOUT>::STAGE +
           (2 * kSurSlots + 2 * kSurRows + 1) * 8 + 32 * 4 + 16;
}

int sur_conv_items(int B, int H, int W, int dil)
{
    const int nsx = (W + 127) / 128;
    const int nch = ((H + dil - 1) / dil + kSurRows - 1) / kSurRows;
    return B * nsx * dil * nch;
}

// 4-D map {32 channels, W, H, B} of a [B][H][W][32] BF16 activation tensor
// (strides 64 B, W*64 B, H*W*64 B) with box {32, box_px, 1, 1} and 64-byte
// swizzle: the conv's input rows (box_px = 128 + 2d) and output tiles
// (box_px = 32).
static int sur_make_map_box(CUtensorMap *tm, const void *act, int B, int H, int W, int box_px)
{
    auto enc = get_encode_fn();
    if (!enc) return fail(GLSU_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[4] = {32, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    cuuint64_t strides[3] = {64, (cuuint64_t)W * 64, (cuuint64_t)H * W * 64};
    cuuint32_t box[4] = {32, (cuuint32_t)box_px, 1, 1};
    cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(act), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(GLSU_ERR_CUDA, "cuTensorMapEncodeTiled failed for an activation map");
    return GLSU_OK;
}

int sur_make_map(CUtensorMap *tm, const void *act, int B, int H, int W, int dil)
{
    if (dil < 1 || 128 + 2 * dil > 256) return fail(GLSU_ERR_INVALID, "surrogate dilation must be 1..64");
    return sur_make_map_box(tm, act, B, H, W, 128 + 2 * dil);
}

int sur_make_out_map(CUtensorMap *tm, const void *act, int B, int H, int W)
{
    return sur_make_map_box(tm, act, B, H, W, 32);
}

template <int NOUT>
static int launch_sur_conv_t(const CUtensorMap &tm, const CUtensorMap &tmo, const SurConvArgs &a, cudaStream_t s)
{
    // registers per thread are a property of the binary (the same on every device)
    static std::atomic<int> regs_cached{0};
    const int smem = sur_conv_smem_bytes<NOUT>(a.dil);
    GLSU_TRY(raise_smem_limit((const void *)sur_conv_tc_kernel<NOUT>, sur_conv_smem_bytes<NOUT>(64),
                              (int)cudaSharedmemCarveoutMaxShared));
    const int sms = device_sm_count();
    int regs = regs_cached.load();
    if (!regs) {
        cudaFuncAttributes fa;
        GLSU_CUDA_TRY(cudaFuncGetAttributes(&fa, sur_conv_tc_kernel<NOUT>));
        regs = std::max(1, fa.numRegs);
        regs_cached.store(regs);
    }
    // persistent: as many CTAs as are resident at once, each walking a
    // strided list of items.  Residency is bounded by registers (per-warp
    // allocation in units of 256), shared memory (1 KB reserved per CTA) and
    // the 512 TMEM columns.
    const int warp_regs = (regs * 32 + 255) / 256 * 256;
    const int by_regs = 65536 / (8 * warp_regs);
    const int by_smem = (228 * 1024) / (smem + 1024);
    const int by_tmem = 512 / SurTc<NOUT>::TMEM_COLS;
    int per_sm = std::max(1, std::min(std::min(by_regs, by_smem), by_tmem));
    if (a.max_ctas_per_sm > 0) per_sm = std::min(per_sm, a.max_ctas_per_sm);
    const int items = sur_conv_items(a.B, a.H, a.W, a.dil);
    const int grid = std::min(items, per_sm * sms);
    sur_conv_tc_kernel<NOUT><<<grid, 256, smem, s>>>(tm, tmo, a, items);
    GLSU_CUDA_TRY(cudaGetLastError());
    return GLSU_OK;
}

int launch_sur_conv(const CUtensorMap &tm, const CUtensorMap &tmo, const SurConvArgs &a, cudaStream_t s)
{
    return launch_sur_conv_t<32>(tm, tmo, a, s);
}

int launch_sur_last(const CUtensorMap &tm, const SurConvArgs &a, cudaStream_t s)
{
    if (!a.z || (!a.cout && !a.yout)) return fail(GLSU_ERR_INVALID, "last surrogate layer without input or output");
    return launch_sur_conv_t<16>(tm, tm, a, s);
}

// ---------------------------------------------------------------------------
// layer 0 (2 -> 32) and layer 7 (32 -> 2) on CUDA cores
// ---------------------------------------------------------------------------
// Layer 0 (2 -> 32, ReLU); z: complex [B][H][W].  The weights are kernel
// parameters, so every FMA takes its weight from the parameter bank.
__global__ void __launch_bounds__(256) sur_l0_kernel(const float2 *__restrict__ z, int B, int H, int W, int dil,
                                                     const __grid_constant__ SurL0W wp, uint16_t *__restrict__ out)
{
    for (int row = blockIdx.x; row < B * H; row += gridDim.x)
        for (int x = threadIdx.x; x < W; x += 256) {
            const int y = row % H;
            const size_t p = (size_t)row * W + x;
            const size_t img = (size_t)(row - y) * W;
            float in[18];
#pragma unroll
            for (int t = 0; t < 9; t++) {
                const int yy = y + (t / 3 - 1) * dil, xx = x + (t % 3 - 1) * dil;
                float2 v = make_float2(0.f, 0.f);
                if (yy >= 0 && yy < H && xx >= 0 && xx < W) v = z[img + (size_t)yy * W + xx];
                in[t] = v.x;
                in[9 + t] = v.y;
            }
            float acc[32];
#pragma unroll
            for (int c = 0; c < 32; c++) {
                float s = wp.b[c];
#pragma unroll
                for (int k = 0; k < 18; k++) s = fmaf(wp.w[c * 18 + k], in[k], s);
                acc[c] = fmaxf(s, 0.f);
            }
            uint4 *op = reinterpret_cast<uint4 *>(out + p * 32);
#pragma unroll
            for (int g = 0; g < 4; g++)
                op[g] = make_uint4(pack_bf2(acc[8 * g], acc[8 * g + 1]), pack_bf2(acc[8 * g + 2], acc[8 * g + 3]),
                                   pack_bf2(acc[8 * g + 4], acc[8 * g + 5]), pack_bf2(acc[8 * g + 6], acc[8 * g + 7]));
        }
}

// Training loss of the last layer's output: from y = z + conv7(a6) (written
// by the tensor-core last layer), out = y / |y| (the same rounding as the
// inference epilogue), per pixel loss wgt |out - t|^2 with wgt =
// min(wscale |target|, 1) and t = target / |target|, the gradient dL/dh7 of
// the mean loss into dh
// and per-block loss sums (fixed order) into part.
__global__ void __launch_bounds__(256) sur_l7_loss_kernel(const float2 *__restrict__ yv,
                                                          const float2 *__restrict__ target, size_t n,
                                                          float2 *__restrict__ out, float2 *__restrict__ dh,
                                                          double *__restrict__ part, float wscale)
{
    __shared__ double red[256];
    const int tid = threadIdx.x;
    const double inv_n = 1.0 / (double)n;
    double lsum = 0;
    for (size_t p = (size_t)blockIdx.x * 256 + tid; p < n; p += (size_t)gridDim.x * 256) {
        const float2 y = yv[p];
        float orr, oii, inv;
        sur_unit(y.x, y.y, orr, oii, inv);
        out[p] = make_float2(orr, oii);
        const float2 tv = target[p];
        const float tn = sqrtf(tv.x * tv.x + tv.y * tv.y);
        const float wgt = fminf(tn * wscale, 1.f);
        const float ti = tn > 1e-20f ? 1.f / tn : 0.f;
        const float er = orr - tv.x * ti, ei = oii - tv.y * ti;
        lsum += (double)(wgt * (er * er + ei * ei)) * inv_n;
        // d out: 2 wgt e / n; through out = y/|y|: (g - out (out.g)) / |y|
        const float gr = (float)(2.0 * inv_n) * wgt * er, gi = (float)(2.0 * inv_n) * wgt * ei;
        const float dot = orr * gr + oii * gi;
        dh[p] = make_float2((gr - orr * dot) * inv, (gi - oii * dot) * inv);
    }
    red[tid] = lsum;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (tid < s) red[tid] += red[tid + s];
        __syncthreads();
    }
    if (tid == 0) part[blockIdx.x] = red[0];
}

// dL/da6 through layer 7, masked by ReLU'(a6): g6[p][ci] = [a6 > 0] *
// sum_t sum_co w7[co][ci][t] dh[p - off_t][co]
__global__ void __launch_bounds__(256) sur_l7_bwd_kernel(const float2 *__restrict__ dh,
                                                         const uint16_t *__restrict__ a6, int B, int H, int W,
                                                         int dil, const float *__restrict__ w7,
                                                         uint16_t *__restrict__ g6)
{
    __shared__ float ws[576];
    for (int e = threadIdx.x; e < 576; e += 256) ws[e] = w7[e];
    __syncthreads();
    for (int row = blockIdx.x; row < B * H; row += gridDim.x)
    for (int x = threadIdx.x; x < W; x += 256) {
        const int y = row % H;
        const size_t p = (size_t)row * W + x;
        const size_t img = (size_t)(row - y) * W;
        float acc[32];
#pragma unroll
        for (int c = 0; c < 32; c++) acc[c] = 0.f;
#pragma unroll
        for (int t = 0; t < 9; t++) {
            const int yy = y - (t / 3 - 1) * dil, xx = x - (t % 3 - 1) * dil;
            if (yy < 0 || yy >= H || xx < 0 || xx >= W) continue;
            const float2 d = dh[img + (size_t)yy * W + xx];
#pragma unroll
            for (int c = 0; c < 32; c++) acc[c] = fmaf(ws[c * 9 + t], d.x, fmaf(ws[288 + c * 9 + t], d.y, acc[c]));
        }
        const uint4 *ap = reinterpret_cast<const uint4 *>(a6 + p * 32);
        uint4 *op = reinterpret_cast<uint4 *>(g6 + p * 32);
#pragma unroll
        for (int g = 0; g < 4; g++) {
            float av[8];
            unpack8(ap[g], av);
#pragma unroll
            for (int i = 0; i < 8; i++)
                if (!(av[i] > 0.f)) acc[8 * g + i] = 0.f;
            op[g] = make_uint4(pack_bf2(acc[8 * g], acc[8 * g + 1]), pack_bf2(acc[8 * g + 2], acc[8 * g + 3]),
                               pack_bf2(acc[8 * g + 4], acc[8 * g + 5]), pack_bf2(acc[8 * g + 6], acc[8 * g + 7]));
        }
    }
}

// ---------------------------------------------------------------------------
// weight gradients
// ---------------------------------------------------------------------------
// 32 -> 32 layer on the tensor cores.  With d the dilation and g the
// gradient w.r.t. the layer's output,
//   dW[co][ci][ky][kx] = sum_{b, y', x} g[b, y' - (ky-1) d, x, co] a[b, y', x + (kx-1) d, ci]
// (y' = y + (ky-1) d: each activation row y' meets the gradient rows y' + d,
// y', y' - d).  A work item is one 128-pixel segment of one activation row.
// Per 16 pixels one MMA D[M = 128][N = 96] += A[M][K = 16] B[K][N]:
//   A: the three gradient rows, M = ky * 32 + co (a zeroed fourth block pads
//      M to 128);
//   B: the activation row, N = kx * 32 + ci, its three kx blocks d pixels
//      apart.
// Both operands are the pixel-major rows that TMA writes with 64-byte
// swizzle, read MN-major: per pixel the 32 channels (64 bytes, the M or N
// direction), pixels 64 bytes apart and 8-pixel groups 512 bytes apart (K),
// the 32-channel blocks LBO apart (the gradient slot stride for A, 64 d bytes
// for B).  The accumulator stays in TMEM across all of a CTA's items; the
// epilogue writes it once as the CTA's partial, part[blk][co][ci][ky*3+kx].
constexpr int kWgStages = 4;
constexpr int kWgSlot = 128 * 64;          // one 128-pixel gradient row segment
constexpr int kWgPad = 16 * 1024;          // slack after the stages
constexpr uint32_t kWgTmemCols = 128;

__host__ __device__ inline int sur_wgrad_act_bytes(int dil) { return ((128 + 2 * dil) * 64 + 1023) & ~1023; }
__host__ __device__ inline int sur_wgrad_stage_bytes(int dil) { return 4 * kWgSlot + sur_wgrad_act_bytes(dil); }
inline int sur_wgrad_smem_bytes(int dil) { return kWgStages * sur_wgrad_stage_bytes(dil) + kWgPad + 256; }

// MN-major operand in the 64-byte swizzle layout: 32-element blocks `lbo`
// bytes apart, 8-row (K) groups 512 bytes apart.
__device__ __forceinline__ uint64_t umma_desc_mn_sw64(uint32_t saddr, uint32_t lbo)
{
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)(512 >> 4) << 32) | ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}

struct SurWgradArgs {
    int B = 0, H = 0, W = 0, dil = 1;
    float *part = nullptr;  // [gridDim.x][9216]
    int *err = nullptr;
};

__global__ void __launch_bounds__(256, 1) sur_wgrad_tc_kernel(const __grid_constant__ CUtensorMap tma,
                                                              const __grid_constant__ CUtensorMap tmg,
                                                              SurWgradArgs a, int nitems)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    const int stage_bytes = sur_wgrad_stage_bytes(a.dil);
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + kWgStages * stage_bytes + kWgPad);
    uint64_t *sfree = full + kWgStages;
    uint64_t *done = sfree + kWgStages;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nsx = (a.W + 127) / 128;
    if (tid == 0) {
        for (int s = 0; s < kWgStages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&sfree[s], 1);
        }
        mbar_init(done, 1);
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(tslot, kWgTmemCols);
    // the fourth gradient block of every stage stays zero: it pads M to 128
    for (int s = 0; s < kWgStages; s++)
        for (int e = tid; e < kWgSlot / 16; e += 256)
            reinterpret_cast<uint4 *>(sm + s * stage_bytes + 3 * kWgSlot)[e] = make_uint4(0, 0, 0, 0);
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0 && lane == 0) {
        // ---- producer: per item three gradient rows and one activation row ----
        uint32_t g = 0;
        bool ok = true;
        for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x, g++) {
            const int sx = item % nsx, yb = item / nsx, y = yb % a.H, b = yb / a.H;
            const int s = g % kWgStages;
            if (g >= (uint32_t)kWgStages && !mbar_wait_bounded(&sfree[s], ((g / kWgStages) - 1) & 1)) {
                ok = false;
                break;
            }
            unsigned char *st = sm + s * stage_bytes;
            mbar_expect_tx(&full[s], 3u * kWgSlot + (uint32_t)(128 + 2 * a.dil) * 64);
            // rows outside the image arrive as zeros
            tma_load_4d(st, &tmg, &full[s], 0, sx * 128, y + a.dil, b);
            tma_load_4d(st + kWgSlot, &tmg, &full[s], 0, sx * 128, y, b);
            tma_load_4d(st + 2 * kWgSlot, &tmg, &full[s], 0, sx * 128, y - a.dil, b);
            tma_load_4d(st + 4 * kWgSlot, &tma, &full[s], 0, sx * 128 - a.dil, y, b);
        }
        if (!ok) atomicExch(a.err, GLSU_ERR_TIMEOUT);
        for (uint32_t j = g > (uint32_t)kWgStages ? g - kWgStages : 0; j < g; j++)
            mbar_wait_bounded(&full[j % kWgStages], (j / kWgStages) & 1);
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        const uint32_t idesc = umma_idesc_bf16(128, 96) | (1u << 15) | (1u << 16);  // A and B MN-major
        uint32_t g = 0, acc = 0;
        bool ok = true;
        for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x, g++) {
            const int s = g % kWgStages;
            if (!mbar_wait_bounded(&full[s], (g / kWgStages) & 1)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t gb = smem_u32(sm + s * stage_bytes), ab = gb + 4 * kWgSlot;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                umma_bf16(tmem, umma_desc_mn_sw64(gb + k * 1024, kWgSlot),
                          umma_desc_mn_sw64(ab + k * 1024, (uint32_t)a.dil * 64), idesc, acc);
                acc = 1;
            }
            umma_commit(&sfree[s]);
        }
        if (!ok) atomicExch(a.err, GLSU_ERR_TIMEOUT);
        umma_commit(done);  // every MMA has completed before the epilogue reads and TMEM is released
        mbar_wait_bounded(done, 0);
    } else if (warp >= 4 && warp < 7) {
        // ---- epilogue: lanes 0-95 (ky = warp - 4, co = lane) -> the CTA's partial ----
        const int ky = warp - 4;
        const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(done, 0));
        if (!ok && lane == 0) atomicExch(a.err, GLSU_ERR_TIMEOUT);
        tc_fence_after();
        const bool any = blockIdx.x < nitems;
        float *pp = a.part + (size_t)blockIdx.x * 9216 + (size_t)lane * 288;
#pragma unroll
        for (int kx = 0; kx < 3; kx++) {
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(ky * 32) << 16) + (uint32_t)(kx * 32), v);
#pragma unroll
            for (int ci = 0; ci < 32; ci++) pp[ci * 9 + ky * 3 + kx] = (any && ok) ? v[ci] : 0.f;
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, kWgTmemCols);
}

int launch_sur_wgrad(const CUtensorMap &tma, const CUtensorMap &tmg, const SurWgradArgs &a, cudaStream_t s,
                     int *nblocks)
{
    if (a.dil < 1 || a.dil > 64) return fail(GLSU_ERR_INVALID, "surrogate dilation must be 1..64");
    GLSU_TRY(raise_smem_limit((const void *)sur_wgrad_tc_kernel, sur_wgrad_smem_bytes(64),
                              (int)cudaSharedmemCarveoutMaxShared));
    const int items = a.B * a.H * ((a.W + 127) / 128);
    const int grid = std::max(1, std::min(items, device_sm_count()));
    sur_wgrad_tc_kernel<<<grid, 256, sur_wgrad_smem_bytes(a.dil), s>>>(tma, tmg, a, items);
    GLSU_CUDA_TRY(cudaGetLastError());
    *nblocks = grid;
    return GLSU_OK;
}

// Bias gradient of a 32-channel layer: part[blk][c] = sum of g[p][c] over
// the block's pixel range.  Thread = (pixel lane 0..63, 8-channel group) with
// 16-byte loads; the 64 lanes' sums are added in lane order.
__global__ void __launch_bounds__(256) sur_db32_kernel(const uint16_t *__restrict__ g, size_t n, int per_block,
                                                       float *__restrict__ part)
{
    __shared__ float s[64][33];
    const int cg = threadIdx.x & 3, pl = threadIdx.x >> 2;
    const size_t p0 = (size_t)blockIdx.x * per_block;
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (size_t p = p0 + pl; p < p0 + per_block && p < n; p += 64) {
        float v[8];
        unpack8(reinterpret_cast<const uint4 *>(g + p * 32)[cg], v);
#pragma unroll
        for (int i = 0; i < 8; i++) acc[i] += v[i];
    }
#pragma unroll
    for (int i = 0; i < 8; i++) s[pl][cg * 8 + i] = acc[i];
    __syncthreads();
    if (threadIdx.x < 32) {
        float t = s[0][threadIdx.x];
        for (int k = 1; k < 64; k++) t += s[k][threadIdx.x];
        part[(size_t)blockIdx.x * 32 + threadIdx.x] = t;
    }
}

// Layer 0 (g: BF16 32 channels, input z: complex) and layer 7 (g = dh:
// complex, input a6: BF16 32 channels) on CUDA cores: a block takes 8 rows
// of one 64-pixel segment, staging per row the gradient and the three input
// rows (with the dilated halo) in shared memory as FP32 (16-byte loads of
// 8 BF16 channels); thread c < 288 owns (tap t = c / 32, j = c % 32) and
// accumulates the two weights that pair j with both channels of the
// 2-channel side.  part[blk][co][ci][t] then the biases part[blk][576 + co].
constexpr int kDsSeg = 64, kDsRows = 8;

__device__ __forceinline__ void store8(float *d, const float *v)
{
    reinterpret_cast<float4 *>(d)[0] = make_float4(v[0], v[1], v[2], v[3]);
    reinterpret_cast<float4 *>(d)[1] = make_float4(v[4], v[5], v[6], v[7]);
}

template <int COUT, int CIN>
__global__ void __launch_bounds__(288) sur_dw_small_kernel(const void *__restrict__ gptr,
                                                           const void *__restrict__ inptr, int B, int H, int W,
                                                           int dil, float *__restrict__ part)
{
    static_assert((COUT == 2 && CIN == 32) || (COUT == 32 && CIN == 2), "layer 0 or layer 7");
    extern __shared__ __align__(16) float dss[];
    const int SW = kDsSeg + 2 * dil;
    float *gs = dss;                      // [64][COUT]
    float *is = gs + kDsSeg * COUT;       // [3][SW][CIN]
    const int nsx = (W + kDsSeg - 1) / kDsSeg, nby = (H + kDsRows - 1) / kDsRows;
    int item = blockIdx.x;
    const int sx = item % nsx;
    item /= nsx;
    const int by = item % nby, b = item / nby;
    const int x0 = sx * kDsSeg;
    const int tid = threadIdx.x, t = tid >> 5, j = tid & 31;
    const int ky = t / 3, kx = t % 3;
    float acc0 = 0.f, acc1 = 0.f, bacc = 0.f;
    const float zero8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int yy = 0; yy < kDsRows; yy++) {
        const int y = by * kDsRows + yy;
        if (y >= H) break;
        __syncthreads();
        if (COUT == 32) {  // g0: 4 x 16 bytes a pixel
            for (int e = tid; e < kDsSeg * 4; e += 288) {
                const int px = e >> 2, c8 = e & 3, x = x0 + px;
                float v[8];
                if (x < W) unpack8(reinterpret_cast<const uint4 *>(gptr)[(((size_t)b * H + y) * W + x) * 4 + c8], v);
                store8(gs + px * 32 + c8 * 8, x < W ? v : zero8);
            }
        } else {  // dh: one complex a pixel
            for (int px = tid; px < kDsSeg; px += 288) {
                const int x = x0 + px;
                float2 v = make_float2(0.f, 0.f);
                if (x < W) v = reinterpret_cast<const float2 *>(gptr)[((size_t)b * H + y) * W + x];
                gs[px * 2] = v.x;
                gs[px * 2 + 1] = v.y;
            }
        }
        if (CIN == 32) {  // a6: 4 x 16 bytes a pixel
            for (int e = tid; e < 3 * SW * 4; e += 288) {
                const int c8 = e & 3, rest = e >> 2, px = rest % SW, r = rest / SW;
                const int ys = y + (r - 1) * dil, xs = x0 - dil + px;
                const bool in = ys >= 0 && ys < H && xs >= 0 && xs < W;
                float v[8];
                if (in) unpack8(reinterpret_cast<const uint4 *>(inptr)[(((size_t)b * H + ys) * W + xs) * 4 + c8], v);
                store8(is + (r * SW + px) * 32 + c8 * 8, in ? v : zero8);
            }
        } else {  // z: one complex a pixel
            for (int e = tid; e < 3 * SW; e += 288) {
                const int px = e % SW, r = e / SW;
                const int ys = y + (r - 1) * dil, xs = x0 - dil + px;
                float2 v = make_float2(0.f, 0.f);
                if (ys >= 0 && ys < H && xs >= 0 && xs < W)
                    v = reinterpret_cast<const float2 *>(inptr)[((size_t)b * H + ys) * W + xs];
                is[(r * SW + px) * 2] = v.x;
                is[(r * SW + px) * 2 + 1] = v.y;
            }
        }
        __syncthreads();
        const float *ir = is + (size_t)(ky * SW + kx * dil) * CIN;
        if (COUT == 2) {  // layer 7: j = ci, the two output channels
#pragma unroll 8
            for (int px = 0; px < kDsSeg; px++) {
                const float iv = ir[px * CIN + j];
                const float2 gv = reinterpret_cast<const float2 *>(gs)[px];
                acc0 = fmaf(gv.x, iv, acc0);
                acc1 = fmaf(gv.y, iv, acc1);
            }
            if (tid < 2)
                for (int px = 0; px < kDsSeg; px++) bacc += gs[px * 2 + tid];
        } else {  // layer 0: j = co, the two input channels
#pragma unroll 8
            for (int px = 0; px < kDsSeg; px++) {
                const float gv = gs[px * 32 + j];
                const float2 iv = reinterpret_cast<const float2 *>(ir)[px];
                acc0 = fmaf(gv, iv.x, acc0);
                acc1 = fmaf(gv, iv.y, acc1);
            }
            if (tid < 32)
                for (int px = 0; px < kDsSeg; px++) bacc += gs[px * 32 + tid];
        }
    }
    float *pp = part + (size_t)blockIdx.x * (COUT * CIN * 9 + COUT);
    if (COUT == 2) {
        pp[(0 * 32 + j) * 9 + t] = acc0;
        pp[(1 * 32 + j) * 9 + t] = acc1;
        if (tid < 2) pp[576 + tid] = bacc;
    } else {
        pp[(j * 2 + 0) * 9 + t] = acc0;
        pp[(j * 2 + 1) * 9 + t] = acc1;
        if (tid < 32) pp[576 + tid] = bacc;
    }
}

int sur_dw_small_blocks(int B, int H, int W)
{
    return B * ((H + kDsRows - 1) / kDsRows) * ((W + kDsSeg - 1) / kDsSeg);
}
int sur_dw_small_smem(int dil, int cout, int cin) { return (kDsSeg * cout + 3 * (kDsSeg + 2 * dil) * cin) * 4; }

// Deterministic column sums of per-block partials: out[c] = sum_b part[b][c].
// A block takes 32 columns; its warps (blockDim.x / 32 of them) sum every
// nw-th partial in FP64, then the warps' sums are added in warp order.
__global__ void __launch_bounds__(1024) sur_reduce_kernel(const float *__restrict__ part, int nblocks, int ncols,
                                                          float *__restrict__ out)
{
    __shared__ double s[32][32];
    const int nw = blockDim.x >> 5, w = threadIdx.x >> 5, l = threadIdx.x & 31;
    const int c = blockIdx.x * 32 + l;
    double acc = 0;
    if (c < ncols)
        for (int b = w; b < nblocks; b += nw) acc += part[(size_t)b * ncols + c];
    s[w][l] = acc;
    __syncthreads();
    if (w == 0 && c < ncols) {
        double t = s[0][l];
        for (int k = 1; k < nw; k++) t += s[k][l];
        out[c] = (float)t;
    }
}

// Threads of a reduction: more warps when there are many partials.
inline int sur_reduce_threads(int nblocks) { return nblocks >= 1024 ? 1024 : nblocks >= 256 ? 512 : 256; }

__global__ void sur_sum_kernel(const double *__restrict__ part, int n, double *__restrict__ out)
{
    double s = 0;
    for (int i = threadIdx.x; i < n; i += 32) s += part[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) *out = s;
}

// ---------------------------------------------------------------------------
// Adam and weight packing
// ---------------------------------------------------------------------------
__global__ void sur_adam_kernel(float *__restrict__ w, const float *__restrict__ grad, float *__restrict__ m,
                                float *__restrict__ v, int n, float lr, float b1, float b2, float eps, float c1,
                                float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = grad[i];
    const float mi = b1 * m[i] + (1 - b1) * gi;
    const float vi = b2 * v[i] + (1 - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

__device__ __forceinline__ float bf16_round(float f) { return __bfloat162float(__float2bfloat16_rn(f)); }

// Element index in the packed B operand (layout of SurTc<NOUT>): tap
// t = 3 dy + dx, K index k (input channel of the layer), N index n (output
// channel): [dx][kc = k / 16][h = (k / 8) % 2][row NOUT (2 - dy) + n][k % 8].
template <int NOUT> __device__ __forceinline__ int sur_bpack_index(int t, int k, int n)
{
    const int dy = t / 3, dx = t % 3;
    return ((dx * 2 + k / 16) * 2 + (k / 8) % 2) * SurTc<NOUT>::BROWS * 8 + (NOUT * (2 - dy) + n) * 8 + k % 8;
}

// From the FP32 master parameters (per layer W[co][ci][3][3] then b[co]):
//   pk_fwd[l] with B[n = co][k = ci] and pk_bwd[l] with B[n = ci][k = co] of
//   the flipped tap 8 - t (the transposed, flipped kernel of the
//   backward-data pass) for the six tensor-core layers; pk7 (if not null,
//   zeroed beforehand) with B[n = co < 2][k = ci] of the last layer; BF16-
//   rounded FP32 copies of layers 0 and 7.
__global__ void sur_pack_kernel(const float *__restrict__ master, uint16_t *__restrict__ pk_fwd,
                                uint16_t *__restrict__ pk_bwd, float *__restrict__ w0r, float *__restrict__ w7r,
                                uint16_t *__restrict__ pk7)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 576) w0r[i] = bf16_round(master[i]);
    const int off7 = kSurL0Params + 6 * kSurL32Params;
    if (i < 576) {
        w7r[i] = bf16_round(master[off7 + i]);
        if (pk7) {
            const __nv_bfloat16 h = __float2bfloat16_rn(master[off7 + i]);
            pk7[sur_bpack_index<16>(i % 9, (i / 9) % 32, i / 288)] = *reinterpret_cast<const uint16_t *>(&h);
        }
    }
    if (i >= 6 * 9216) return;
    const int l = i / 9216, e = i % 9216;
    const int co = e / 288, ci = (e / 9) % 32, t = e % 9;
    const float wv = master[kSurL0Params + l * kSurL32Params + e];
    const __nv_bfloat16 h = __float2bfloat16_rn(wv);
    const uint16_t bits = *reinterpret_cast<const uint16_t *>(&h);
    // forward: B[n = 32 (2 - dy) + co][k = ci] of tap t = 3 dy + dx
    pk_fwd[(size_t)l * 9216 + sur_bpack_index<32>(t, ci, co)] = bits;
    // backward data: B[n = 32 (2 - dy') + ci][k = co] of the flipped tap t' = 8 - t
    pk_bwd[(size_t)l * 9216 + sur_bpack_index<32>(8 - t, co, ci)] = bits;
}

// Gather training crops: x[b] = pool_x[idx[b]][oy:oy+h, ox:ox+w] (complex),
// same for the target.  The crop list travels as a kernel parameter, so a
// step needs no copy and no synchronisation.
constexpr int kSurMaxBatch = 512;
struct SurCrops {
    int4 c[kSurMaxBatch];  // (pool index, oy, ox, unused)
};

__global__ void sur_gather_kernel(const float2 *__restrict__ px, const float2 *__restrict__ pt, int PH, int PW,
                                  const __grid_constant__ SurCrops crops, int B, int h, int w,
                                  float2 *__restrict__ x, float2 *__restrict__ t)
{
    const size_t n = (size_t)B * h * w;
    for (size_t p = (size_t)blockIdx.x * 256 + threadIdx.x; p < n; p += (size_t)gridDim.x * 256) {
        const int xx = (int)(p % w), yy = (int)((p / w) % h), b = (int)(p / ((size_t)w * h));
        const int4 c = crops.c[b];
        const size_t src = ((size_t)c.x * PH + c.y + yy) * PW + c.z + xx;
        x[p] = px[src];
        t[p] = pt[src];
    }
}

}  // namespace glsu
