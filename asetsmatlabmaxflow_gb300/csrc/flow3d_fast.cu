// Compiled instances of the fused iteration kernel for the labelled models (divergence
// epilogue), 3D tiles 28 x 28, 28 x 12, 28 x 8; fast projection, built with FMA
// contraction and flush to zero (held to the parity tolerance, not bit-exactness).
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    // default: the fewest halo threads; the plane loop unrolled by 4, the
    // refill issued in Z by the producer's halo-column warp
    make_variant<3, 32, 4, EPI_DIV, false, 1, 4, 1, true>(),
    make_variant<3, 16, 6, EPI_DIV, false, 1, 4, 1, true>(),  // 28 x 12, six stages (large volumes)
    make_variant<3, 16, 4, EPI_DIV, false>(),
    make_variant<3, 12, 4, EPI_DIV, false>(),
    make_variant<3, 12, 8, EPI_DIV, false, 2, 4, 1, true>(),   // 28 x 8, eight stages (small volumes)
    make_variant<3, 16, 8, EPI_DIV, false, 1, 4, 1, true>(),   // 28 x 12, eight stages
};

const StencilVariant *flow3d_fast_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
