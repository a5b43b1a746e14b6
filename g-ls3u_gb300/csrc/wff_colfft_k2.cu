// wff_colfft_k2.cu -- FFT column sweep kernels for transform lengths 1024 and 1280.
#include "wff_colfft_plans.cuh"

namespace glsu {
namespace colfft {
int launch_len_mid(int L, int ncol, const WffPlan &Pl, cudaStream_t s, const int2 *list, const int *count,
                   int grid_x)
{
    switch (L) {
        GLSU_COLFFT_CASE(1024, P1024, 4)
        GLSU_COLFFT_CASE(1280, P1280, 4)
    default: return GLSU_ERR_UNSUPPORTED;
    }
}
int launch_batch_mid(int L, const BatchTable &tab, int nseq, int nitems, const float2 *tw, int grid_x, cudaStream_t s)
{
    switch (L) {
        GLSU_COLFFT_BATCH_CASE(1024, P1024, 4)
        GLSU_COLFFT_BATCH_CASE(1280, P1280, 4)
    default: return GLSU_ERR_UNSUPPORTED;
    }
}
}  // namespace colfft
}  // namespace glsu
