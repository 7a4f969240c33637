// Compiled instances of the fused iteration kernel for the labelled models (divergence
// epilogue), 2D tiles 240-row (two rows per thread), 224-row, 56-row; fast
// projection, built with FMA contraction and flush to zero (held to the parity
// tolerance, not bit-exactness).
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    // default: two rows per thread, 240-row tiles, 4 stages, the plane loop
    // unrolled by 4
    make_variant<2, 4, 4, EPI_DIV, false, 4, 4, 2>(),
    make_variant<2, 8, 4, EPI_DIV, false, 4, 4>(),       // 224-row tiles
    make_variant<2, 2, 4, EPI_DIV, false>(),             // 56-row tiles (short columns)
    make_variant<2, 4, 6, EPI_DIV, false, 4, 4, 2>(),
};

const StencilVariant *flow2d_fast_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
