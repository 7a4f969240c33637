// Compiled instances of the fused iteration kernel for the labelled models (divergence
// epilogue), 3D tiles 28 x 28, 28 x 12, 28 x 8; EXACT projection, built with the reference's
// float arithmetic (no FMA contraction, no flush to zero).
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    // the fast defaults' geometries: 28 x 28 unrolled by 4 with the refill
    // in Z, 28 x 12 with six stages, and eight-stage rings for small volumes
    make_variant<3, 32, 4, EPI_DIV, true, 1, 4, 1, true>(),
    make_variant<3, 16, 6, EPI_DIV, true, 1, 4, 1, true>(),
    make_variant<3, 16, 4, EPI_DIV, true>(),
    make_variant<3, 12, 4, EPI_DIV, true>(),
    make_variant<3, 12, 8, EPI_DIV, true, 2, 4, 1, true>(),
    make_variant<3, 16, 8, EPI_DIV, true, 1, 4, 1, true>(),
};

const StencilVariant *flow3d_exact_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
