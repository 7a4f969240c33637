// Compiled instances of the fused iteration kernel for the binary model (ps/pt/u
// epilogue), 3D tiles 60 x 12 and 60 x 16 (two rows per thread), 28 x 28, 28 x 12, 28 x 8;
// fast projection, built with FMA
// contraction and flush to zero (held to the parity tolerance, not bit-exactness).
#include "variants.cuh"

namespace asets {

static const StencilVariant kVariants[] = {
    // default: two rows per thread (60 x 12 tiles, 512 threads), a ring of
    // five stages, the plane loop unrolled by 8, the refill issued in Z by
    // the producer's halo-column warp
    make_variant<3, 16, 5, EPI_BINARY, false, 1, 8, 2, true>(),
    make_variant<3, 20, 4, EPI_BINARY, false, 1, 4, 2, true>(),   // 60 x 16, four stages
    // one row per thread: 28 x 28 tiles, the fewest halo threads
    make_variant<3, 32, 4, EPI_BINARY, false, 1, 4>(),
    make_variant<3, 16, 4, EPI_BINARY, false>(),
    make_variant<3, 12, 4, EPI_BINARY, false>(),
};

const StencilVariant *binary3d_fast_variants(int *count)
{
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace asets
