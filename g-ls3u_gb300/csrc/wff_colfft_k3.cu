// wff_colfft_k3.cu -- FFT column sweep kernels for transform lengths 1536 .. 4096.
#include "wff_colfft_plans.cuh"

namespace glsu {
namespace colfft {
int launch_len_large(int L, int ncol, const WffPlan &Pl, cudaStream_t s, const int2 *list, const int *count,
                     int grid_x)
{
    switch (L) {
        GLSU_COLFFT_CASE(1536, P1536, 2)
        GLSU_COLFFT_CASE(2048, P2048, 2)
        GLSU_COLFFT_CASE(2560, P2560, 2)
        GLSU_COLFFT_CASE(3072, P3072, 1)
        GLSU_COLFFT_CASE(4096, P4096, 1)
    default: return GLSU_ERR_UNSUPPORTED;
    }
}
int launch_batch_large(int L, const BatchTable &tab, int nseq, int nitems, const float2 *tw, int grid_x, cudaStream_t s)
{
    switch (L) {
        GLSU_COLFFT_BATCH_CASE(1536, P1536, 2)
        GLSU_COLFFT_BATCH_CASE(2048, P2048, 2)
        GLSU_COLFFT_BATCH_CASE(2560, P2560, 2)
        GLSU_COLFFT_BATCH_CASE(3072, P3072, 1)
        GLSU_COLFFT_BATCH_CASE(4096, P4096, 1)
    default: return GLSU_ERR_UNSUPPORTED;
    }
}
}  // namespace colfft
}  // namespace glsu
