// Compiled instances of the fused iteration kernel for the binary model (ps/pt/u
// epilogue), 3D tiles 60 x 12 and 60 x 16 (two rows per thread), 28 x 12, 28 x 8;
// EXACT projection, built with the reference's
// float arithmetic (no FMA contraction, no flush to zero).
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    // the geometry of the fast default: two rows per thread (60 x 12 tiles),
    // five stages, the plane loop unrolled by 8, the refill issued in Z
    make_variant<3, 16, 5, EPI_BINARY, true, 1, 8, 2, true>(),
    make_variant<3, 20, 4, EPI_BINARY, true, 1, 4, 2, true>(),   // 60 x 16, four stages
    make_variant<3, 16, 4, EPI_BINARY, true>(),
    make_variant<3, 12, 4, EPI_BINARY, true>(),
};

const StencilVariant *binary3d_exact_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
