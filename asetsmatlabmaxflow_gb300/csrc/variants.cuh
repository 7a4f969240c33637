// Helper that turns one stencil_col_kernel instance into a table entry.
#pragma once

#include "internal.h"
#include "stencil2_kernel.cuh"

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
    v.fn = reinterpret_cast<const void *>(&stencil_col_kernel<DIM, NW, NSTAGE, EPI, EXACT, MINB, UNROLL, CELLS, LATE>);
    return v;
}

}  // namespace asets
