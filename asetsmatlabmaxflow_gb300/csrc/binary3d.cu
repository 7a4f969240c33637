// Compiled instances of the fused iteration kernel: 3D tiles 32x16 (2 blocks/SM) and 32x8 (3 blocks/SM),
// fast and EXACT projection.
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    make_variant<3, 32, 16, 256, 3, EPI_BINARY, false>(),
    make_variant<3, 32, 16, 256, 3, EPI_BINARY, true>(),
    make_variant<3, 32, 8, 256, 4, EPI_BINARY, false>(),
    make_variant<3, 32, 8, 256, 4, EPI_BINARY, true>(),
};

const StencilVariant *binary3d_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
