// Compiled instances of the fused iteration kernel for the labelled models (divergence
// epilogue), 3D tiles 28 x 12, 28 x 8; EXACT projection, built with the reference's
// float arithmetic (no FMA contraction, no flush to zero).
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    make_variant<3, 16, 4, EPI_DIV, true>(),
    make_variant<3, 12, 4, EPI_DIV, true>(),
};

const StencilVariant *flow3d_exact_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
