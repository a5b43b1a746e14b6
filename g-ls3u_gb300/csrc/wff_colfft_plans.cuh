// wff_colfft_plans.cuh -- the compiled transform lengths of the FFT column
// sweep: L = radices (radix 8 first, the one radix 3 or 5 last), threads per
// column T, default columns per CTA (4 warps a CTA).
#pragma once
#include "wff_colfft.cuh"

namespace glsu {
namespace colfft {
using P256 = Plan<256, 32, 8, 8, 4>;
using P384 = Plan<384, 16, 8, 8, 2, 3>;
using P512 = Plan<512, 32, 8, 8, 8>;
using P640 = Plan<640, 16, 8, 8, 2, 5>;
using P768 = Plan<768, 32, 8, 8, 4, 3>;
using P1024 = Plan<1024, 32, 8, 8, 4, 4>;
using P1280 = Plan<1280, 32, 8, 8, 4, 5>;
using P1536 = Plan<1536, 64, 8, 8, 8, 3>;
using P2048 = Plan<2048, 64, 8, 8, 8, 4>;
using P2560 = Plan<2560, 64, 8, 8, 8, 5>;
using P3072 = Plan<3072, 128, 8, 8, 4, 4, 3>;
using P4096 = Plan<4096, 128, 8, 8, 8, 8>;
}  // namespace colfft
}  // namespace glsu
