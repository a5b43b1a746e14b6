// dpra_ls_tiles.cu -- the float-float DPRA least squares with the output
// tiles other than the default 32 x 16: tile 1 = 32 x 8 (256 threads, three
// CTAs per SM at r = 3), tile 2 = 32 x 32 (1024 threads, less halo: 1.41
// against 1.63 input elements per output at r = 3).
#include "dpra_ls_ff.cuh"

namespace glsu {

template <int TX, int TY>
static int launch_tile(int img_type, const void *d_img, const void *d_phiref, void *d_z, int W, int H, int r,
                       cudaStream_t s)
{
#define GLSU_TILE_R(RR)                                                                                  \
    case RR:                                                                                             \
        return img_type == GLSU_U8                                                                       \
                   ? launch_ff_tile<uint8_t, RR, TX, TY>(d_img, d_phiref, d_z, W, H, s)                  \
                   : launch_ff_tile<float, RR, TX, TY>(d_img, d_phiref, d_z, W, H, s);
    if (img_type != GLSU_U8 && img_type != GLSU_F32) return fail(GLSU_ERR_INVALID, "unsupported frame type");
    switch (r) {
        GLSU_TILE_R(1)
        GLSU_TILE_R(2)
        GLSU_TILE_R(3)
        GLSU_TILE_R(4)
        GLSU_TILE_R(5)
        GLSU_TILE_R(6)
        GLSU_TILE_R(7)
        GLSU_TILE_R(8)
    default: return fail(GLSU_ERR_UNSUPPORTED, "DPRA window radius must be 1..8");
    }
#undef GLSU_TILE_R
}

size_t dpra_ls_ff_smem(int tx, int ty, int r) { return ff_ls_smem_bytes(tx, ty, r); }

int launch_dpra_ls_ff_tile(int tile, int img_type, const void *d_img, const void *d_phiref, void *d_z, int W, int H,
                           int r, cudaStream_t s)
{
    if (tile == 1) return launch_tile<32, 8>(img_type, d_img, d_phiref, d_z, W, H, r, s);
    if (tile == 2) return launch_tile<32, 32>(img_type, d_img, d_phiref, d_z, W, H, r, s);
    return fail(GLSU_ERR_INVALID, "unknown least-squares tile");
}

}  // namespace glsu
