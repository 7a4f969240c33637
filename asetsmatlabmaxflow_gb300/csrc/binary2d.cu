// Compiled instances of the fused iteration kernel: 2D row tiles of 224 (8 warps) and 56 (2 warps),
// fast and EXACT projection.
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    make_variant<2, 8, 4, EPI_BINARY, false>(),
    make_variant<2, 8, 4, EPI_BINARY, true>(),
    make_variant<2, 2, 4, EPI_BINARY, false>(),
    make_variant<2, 2, 4, EPI_BINARY, true>(),
};

const StencilVariant *binary2d_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
