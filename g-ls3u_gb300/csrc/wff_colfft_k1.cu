// wff_colfft_k1.cu -- FFT column sweep kernels for transform lengths 256 .. 768.
#include "wff_colfft_plans.cuh"

namespace glsu {
namespace colfft {
int launch_len_small(int L, int ncol, const WffPlan &Pl, cudaStream_t s, const int2 *list, const int *count,
                     int grid_x)
{
    switch (L) {
        GLSU_COLFFT_CASE(256, P256, 4)
        GLSU_COLFFT_CASE(384, P384, 8)
        GLSU_COLFFT_CASE(512, P512, 4)
        GLSU_COLFFT_CASE(640, P640, 8)
        GLSU_COLFFT_CASE(768, P768, 4)
    default: return GLSU_ERR_UNSUPPORTED;
    }
}
int launch_batch_small(int L, const BatchTable &tab, int nseq, int nitems, const float2 *tw, int grid_x, cudaStream_t s)
{
    switch (L) {
        GLSU_COLFFT_BATCH_CASE(256, P256, 4)
        GLSU_COLFFT_BATCH_CASE(384, P384, 8)
        GLSU_COLFFT_BATCH_CASE(512, P512, 4)
        GLSU_COLFFT_BATCH_CASE(640, P640, 8)
        GLSU_COLFFT_BATCH_CASE(768, P768, 4)
    default: return GLSU_ERR_UNSUPPORTED;
    }
}
}  // namespace colfft
}  // namespace glsu
