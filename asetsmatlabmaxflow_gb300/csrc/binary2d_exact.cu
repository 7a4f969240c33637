// Compiled instances of the fused iteration kernel for the binary model (ps/pt/u
// epilogue), 2D tiles 240-row (two rows per thread), 224-row, 56-row, and two
// iterations per pass with 224-row tiles; EXACT projection, built with the reference's
// float arithmetic (no FMA contraction, no flush to zero).
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    // two rows per thread, 240-row tiles, 6 stages, unrolled by 4
    make_variant<2, 4, 6, EPI_BINARY, true, 4, 4, 2>(),
    make_variant<2, 8, 4, EPI_BINARY, true>(),
    make_variant<2, 2, 4, EPI_BINARY, true>(),
    // two iterations per pass, 224-row tiles
    make_variant_t2<4, 5, true, 3, 4>(),
    // square tiles for small images: 32 x 32 (256 threads), 16 x 16 (128)
    make_variant_tile<32, 32, 256, true>(),
    make_variant_tile<16, 16, 128, true, 4>(),
    // the same, every iteration in one cooperative launch (single solves)
    make_variant_tile<32, 32, 256, true, 2, true>(),
    make_variant_tile<16, 16, 128, true, 4, true>(),
};

const StencilVariant *binary2d_exact_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
