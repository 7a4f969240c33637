// Compiled instances of the one-pass multi-label 2D kernels (stencil2d_labels.cuh)
// for the Ishikawa model, 2 to 9 labels: the label update in the flow
// warps, by one label warp, by two; and the 16 x 16 tile kernels (any label
// count); EXACT projection, built with the reference's float arithmetic (no
// FMA contraction, no flush to zero).
#include "variants.cuh"

namespace asets {

static const StencilVariant kSync[] = {
    make_variant_labels<2, 2, true, 0>(),
    make_variant_labels<2, 3, true, 0>(),
    make_variant_labels<2, 4, true, 0>(),
    make_variant_labels<2, 5, true, 0>(),
    make_variant_labels<2, 6, true, 0>(),
    make_variant_labels<2, 7, true, 0>(),
    make_variant_labels<2, 8, true, 0>(),
    make_variant_labels<2, 9, true, 0>(),
};
static const StencilVariant kOne[] = {
    make_variant_labels<2, 2, true, 1>(),
    make_variant_labels<2, 3, true, 1>(),
    make_variant_labels<2, 4, true, 1>(),
    make_variant_labels<2, 5, true, 1>(),
    make_variant_labels<2, 6, true, 1>(),
    make_variant_labels<2, 7, true, 1>(),
    make_variant_labels<2, 8, true, 1>(),
    make_variant_labels<2, 9, true, 1>(),
};
static const StencilVariant kTwo[] = {
    make_variant_labels<2, 2, true, 2>(),
    make_variant_labels<2, 3, true, 2>(),
    make_variant_labels<2, 4, true, 2>(),
    make_variant_labels<2, 5, true, 2>(),
    make_variant_labels<2, 6, true, 2>(),
    make_variant_labels<2, 7, true, 2>(),
    make_variant_labels<2, 8, true, 2>(),
    make_variant_labels<2, 9, true, 2>(),
};

// 16 x 16 tiles, any label count: one launch per iteration, whole solve
static const StencilVariant kTiles[] = {
    make_variant_tile_labels<2, true, false>(),
    make_variant_tile_labels<2, true, true>(),
};

// the instance for nlab labels (which: 0 in-step update, 1 one label warp,
// 2 two, 3 16 x 16 tiles, 4 16 x 16 tiles for the whole solve), or null
const StencilVariant *ishikawa2d_fused_exact_variant(int nlab, int which)
{
    const int i = nlab - 2;
    if (i < 0 || i >= (int)(sizeof(kOne) / sizeof(kOne[0])) || which < 0 || which > 4)
        return nullptr;
    if (which >= 3)
        return &kTiles[which - 3];
    return which == 0 ? &kSync[i] : which == 1 ? &kOne[i] : &kTwo[i];
}

}  // namespace asets
