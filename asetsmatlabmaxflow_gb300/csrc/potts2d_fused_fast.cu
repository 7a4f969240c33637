// Compiled instances of the one-pass multi-label 2D kernels (stencil2d_labels.cuh)
// for the Potts model, 1 to 8 labels: the label update in the flow
// warps, by one label warp, by two; and the 16 x 16 tile kernels (any label
// count); fast projection, built with FMA contraction and flush to zero
// (held to the parity tolerance, not bit-exactness).
#include "variants.cuh"

namespace asets {

static const StencilVariant kSync[] = {
    make_variant_labels<1, 1, false, 0>(),
    make_variant_labels<1, 2, false, 0>(),
    make_variant_labels<1, 3, false, 0>(),
    make_variant_labels<1, 4, false, 0>(),
    make_variant_labels<1, 5, false, 0>(),
    make_variant_labels<1, 6, false, 0>(),
    make_variant_labels<1, 7, false, 0>(),
    make_variant_labels<1, 8, false, 0>(),
};
static const StencilVariant kOne[] = {
    make_variant_labels<1, 1, false, 1>(),
    make_variant_labels<1, 2, false, 1>(),
    make_variant_labels<1, 3, false, 1>(),
    make_variant_labels<1, 4, false, 1>(),
    make_variant_labels<1, 5, false, 1>(),
    make_variant_labels<1, 6, false, 1>(),
    make_variant_labels<1, 7, false, 1>(),
    make_variant_labels<1, 8, false, 1>(),
};
static const StencilVariant kTwo[] = {
    make_variant_labels<1, 1, false, 2>(),
    make_variant_labels<1, 2, false, 2>(),
    make_variant_labels<1, 3, false, 2>(),
    make_variant_labels<1, 4, false, 2>(),
    make_variant_labels<1, 5, false, 2>(),
    make_variant_labels<1, 6, false, 2>(),
    make_variant_labels<1, 7, false, 2>(),
    make_variant_labels<1, 8, false, 2>(),
};

// 16 x 16 tiles, any label count: one launch per iteration, whole solve
static const StencilVariant kTiles[] = {
    make_variant_tile_labels<1, false, false>(),
    make_variant_tile_labels<1, false, true>(),
};

// the instance for nlab labels (which: 0 in-step update, 1 one label warp,
// 2 two, 3 16 x 16 tiles, 4 16 x 16 tiles for the whole solve), or null
const StencilVariant *potts2d_fused_fast_variant(int nlab, int which)
{
    const int i = nlab - 1;
    if (i < 0 || i >= (int)(sizeof(kOne) / sizeof(kOne[0])) || which < 0 || which > 4)
        return nullptr;
    if (which >= 3)
        return &kTiles[which - 3];
    return which == 0 ? &kSync[i] : which == 1 ? &kOne[i] : &kTwo[i];
}

}  // namespace asets
