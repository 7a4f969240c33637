// Compiled instances of the fused iteration kernels for the binary model (ps/pt/u
// epilogue), 2D: two iterations per pass with 224-row tiles (default), one
// iteration per pass with 240-row (two rows per thread), 224-row and 56-row
// tiles; fast projection, built with FMA contraction and flush to zero (held
// to the parity tolerance, not bit-exactness).
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    // default: two iterations per pass (stencil2d_t2.cuh), 224-row tiles,
    // five stages, the plane loop unrolled by 4
    make_variant_t2<4, 5, false, 3, 4>(),
    // one iteration per pass: two rows per thread, 240-row tiles, 6 stages,
    // the plane loop unrolled by 4
    make_variant<2, 4, 6, EPI_BINARY, false, 4, 4, 2>(),
    make_variant<2, 8, 4, EPI_BINARY, false, 4, 4>(),       // 224-row tiles
    make_variant<2, 2, 4, EPI_BINARY, false>(),             // 56-row tiles (short columns)
    make_variant<2, 4, 4, EPI_BINARY, false, 4, 4, 2>(),
    // square tiles for small images: 32 x 32 (256 threads), 16 x 16 (128)
    make_variant_tile<32, 32, 256, false>(),
    make_variant_tile<16, 16, 128, false, 4>(),
    // the same, every iteration in one cooperative launch (single solves)
    make_variant_tile<32, 32, 256, false, 2, true>(),
    make_variant_tile<16, 16, 128, false, 4, true>(),
};

const StencilVariant *binary2d_fast_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
