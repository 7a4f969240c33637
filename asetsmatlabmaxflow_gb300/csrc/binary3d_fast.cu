// Compiled instances of the fused iteration kernel for the binary model (ps/pt/u
// epilogue), 3D tiles 28 x 28, 28 x 12, 28 x 8; fast projection, built with FMA
// contraction and flush to zero (held to the parity tolerance, not bit-exactness).
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    make_variant<3, 32, 4, EPI_BINARY, false, 1>(),  // default: the fewest halo threads
    make_variant<3, 16, 4, EPI_BINARY, false>(),
    make_variant<3, 12, 4, EPI_BINARY, false>(),
};

const StencilVariant *binary3d_fast_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
