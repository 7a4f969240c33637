// Helper that turns one stencil_col_kernel instance into a table entry.
#pragma once

#include "internal.h"
#include "stencil2_kernel.cuh"
#include "stencil2d_t2.cuh"
#include "stencil2d_labels.cuh"
#include "stencil2d_tile.cuh"
#include "stencil2d_tile_labels.cuh"

namespace asets {

template <int DIM, int NW, int NSTAGE, int EPI, bool EXACT, int MINB = (DIM == 3 ? 2 : 4),
          int UNROLL = 1, int CELLS = 1, bool LATE = false>
StencilVariant make_variant()
{
    using G = ColGeom<DIM, NW, CELLS>;
    StencilVariant v;
    v.dim = DIM;
    v.epi = EPI;
    v.exact = EXACT ? 1 : 0;
    v.tr = G::TR;
    v.tc = G::TC;
    v.nt = G::NT;
    v.nstage = NSTAGE;
    v.smem_bytes = G::template smem_bytes<NSTAGE, EPI>();
    v.box_rows = G::LR;
    v.box_cols = G::LC;
    v.box_cols_bc = G::LC_BC;
    v.tile_box_rows = G::TR;
    v.temporal = 1;
    v.fn = reinterpret_cast<const void *>(&stencil_col_kernel<DIM, NW, NSTAGE, EPI, EXACT, MINB, UNROLL, CELLS, LATE>);
    return v;
}

// The binary 2D kernel with two iterations per pass (stencil2d_t2.cuh).
template <int NW, int NSTAGE, bool EXACT, int MINB, int UNROLL>
StencilVariant make_variant_t2()
{
    using G = T2Geom<NW>;
    StencilVariant v;
    v.dim = 2;
    v.epi = EPI_BINARY;
    v.exact = EXACT ? 1 : 0;
    v.tr = G::TR;
    v.tc = 1;
    v.nt = G::NT;
    v.nstage = NSTAGE;
    v.smem_bytes = G::template smem_bytes<NSTAGE>();
    v.box_rows = G::LR;
    v.box_cols = 1;
    v.box_cols_bc = 1;
    v.tile_box_rows = G::TB;
    v.temporal = 2;
    v.fn = reinterpret_cast<const void *>(&stencil2d_t2_kernel<NW, NSTAGE, EXACT, MINB, UNROLL>);
    return v;
}

// The binary 2D square-tile kernels (stencil2d_tile.cuh): R x S tiles, NT
// threads; one launch per iteration, or (PERSISTENT) every iteration in one
// cooperative launch.
template <int R, int S, int NT, bool EXACT, int MINB = 2, bool PERSISTENT = false>
StencilVariant make_variant_tile()
{
    using G = Tile2Geom<R, S>;
    StencilVariant v;
    v.dim = 2;
    v.epi = EPI_BINARY;
    v.exact = EXACT ? 1 : 0;
    v.tr = R;
    v.tc = 1;
    v.nt = NT;
    v.nstage = 0;
    v.smem_bytes = G::smem_bytes();
    v.box_rows = R + 8;       // unused maps, encoded like the sweep's
    v.box_cols = 1;
    v.box_cols_bc = 1;
    v.tile_box_rows = R;
    v.temporal = 1;
    if constexpr (PERSISTENT)
        v.fn = reinterpret_cast<const void *>(&stencil2d_tile_persistent_kernel<R, S, NT, EXACT, MINB>);
    else
        v.fn = reinterpret_cast<const void *>(&stencil2d_tile_kernel<R, S, NT, EXACT, MINB>);
    v.s_tile = S;
    v.persistent = PERSISTENT ? 1 : 0;
    return v;
}

// The multi-label 2D 16 x 16 tile kernels (stencil2d_tile_labels.cuh) for
// MODEL (1 Potts, 2 Ishikawa), any label count up to 8 flow labels, four
// label groups of 128 threads; one launch per iteration, or (PERSISTENT) the
// whole solve in one cooperative launch.  pt/u/ps ping-pong as in the
// one-pass sweep kernels; shared memory sized per launch by label count.
template <int MODEL, bool EXACT, bool PERSISTENT>
StencilVariant make_variant_tile_labels()
{
    using G = LTileGeom<MODEL>;
    constexpr int NT = G::NT;
    StencilVariant v;
    v.dim = 2;
    v.epi = EPI_FUSED;
    v.exact = EXACT ? 1 : 0;
    v.tr = G::R;
    v.tc = 1;
    v.nt = NT;
    v.nstage = 0;
    v.smem_bytes = G::smem_base();
    v.smem_per_fl = G::smem_per_fl();
    v.smem_per_l = G::smem_per_l();
    v.box_rows = G::R + 8;    // unused maps, encoded like the sweep's
    v.box_cols = 1;
    v.box_cols_bc = 1;
    v.tile_box_rows = G::R;
    v.temporal = 1;
    if constexpr (PERSISTENT)
        v.fn = reinterpret_cast<const void *>(&stencil2d_tile_labels_persistent_kernel<MODEL, NT, EXACT>);
    else
        v.fn = reinterpret_cast<const void *>(&stencil2d_tile_labels_kernel<MODEL, NT, EXACT>);
    v.s_tile = G::S;
    v.persistent = PERSISTENT ? 1 : 0;
    return v;
}

// The one-pass multi-label 2D kernels (stencil2d_labels.cuh) for MODEL
// (1 Potts, 2 Ishikawa) with L labels: one warp per flow label, and LW label
// warps (1 or 2; 0: the label update in the flow warps), about 768 threads
// per SM.
template <int MODEL, int L, bool EXACT, int LW, int NSTAGE = 4>
StencilVariant make_variant_labels()
{
    using G = Lab2Geom<MODEL, L>;
    constexpr int NW = G::FL + LW;
    constexpr int MINB = (24 / NW < 1) ? 1 : (24 / NW > 16 ? 16 : 24 / NW);
    StencilVariant v;
    v.dim = 2;
    v.epi = EPI_FUSED;
    v.exact = EXACT ? 1 : 0;
    v.tr = G::TR;
    v.tc = 1;
    v.nt = 32 * NW;
    v.nstage = NSTAGE;
    if constexpr (LW == 0) {
        v.smem_bytes = Lab2SyncGeom<MODEL, L>::template smem_bytes<NSTAGE>();
        v.fn = reinterpret_cast<const void *>(
            &stencil2d_labels_sync_kernel<MODEL, L, NSTAGE, EXACT, MINB>);
    } else {
        v.smem_bytes = Lab2WarpsGeom<MODEL, L, LW>::template smem_bytes<NSTAGE>();
        v.fn = reinterpret_cast<const void *>(
            &stencil2d_labels_kernel<MODEL, L, LW, NSTAGE, EXACT, MINB>);
    }
    v.box_rows = G::LR;
    v.box_cols = 1;
    v.box_cols_bc = 1;
    v.tile_box_rows = G::TR;
    v.temporal = 1;
    v.label_boxes = LB_ALL;
    v.ct_box_rows = G::LR;
    return v;
}

}  // namespace asets
