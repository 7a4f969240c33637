// Compiled instances of the fused iteration kernel: 2D row tiles of 128 and 32,
// fast and EXACT projection.
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    make_variant<2, 128, 1, 160, 4, EPI_BINARY, false>(),
    make_variant<2, 128, 1, 160, 4, EPI_BINARY, true>(),
    make_variant<2, 32, 1, 64, 4, EPI_BINARY, false>(),
    make_variant<2, 32, 1, 64, 4, EPI_BINARY, true>(),
};

const StencilVariant *binary2d_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
