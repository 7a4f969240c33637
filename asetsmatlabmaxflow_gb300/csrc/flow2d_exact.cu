// Compiled instances of the fused iteration kernel for the labelled models (divergence
// epilogue), 2D tiles 240-row (two rows per thread), 224-row, 56-row; EXACT projection,
// built with the reference's float arithmetic (no FMA contraction, no flush to zero).
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    // two rows per thread, 240-row tiles (four and six stages)
    make_variant<2, 4, 4, EPI_DIV, true, 4, 4, 2>(),
    make_variant<2, 8, 4, EPI_DIV, true>(),
    make_variant<2, 2, 4, EPI_DIV, true>(),
    make_variant<2, 4, 6, EPI_DIV, true, 4, 4, 2>(),
};

const StencilVariant *flow2d_exact_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
