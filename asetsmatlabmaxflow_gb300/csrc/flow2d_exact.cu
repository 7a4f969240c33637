// Compiled instances of the fused iteration kernel for the labelled models (divergence
// epilogue), 2D tiles 224-row, 56-row; EXACT projection, built with the reference's
// float arithmetic (no FMA contraction, no flush to zero).
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    make_variant<2, 8, 4, EPI_DIV, true>(),
    make_variant<2, 2, 4, EPI_DIV, true>(),
};

const StencilVariant *flow2d_exact_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
