// Compiled instances of the fused iteration kernel: 3D tiles of 28 x 12 (16 warps) and 28 x 8 (12 warps),
// fast and EXACT projection.
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    make_variant<3, 16, 4, EPI_DIV, false>(),
    make_variant<3, 16, 4, EPI_DIV, true>(),
    make_variant<3, 12, 4, EPI_DIV, false>(),
    make_variant<3, 12, 4, EPI_DIV, true>(),
};

const StencilVariant *flow3d_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
