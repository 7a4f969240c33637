// Helper that turns one stencil_iteration_kernel instance into a table entry.
#pragma once

#include "internal.h"
#include "stencil_kernel.cuh"

namespace asets {

template <int DIM, int TR, int TC, int NT, int NSTAGE, int EPI, bool EXACT>
StencilVariant make_variant()
{
    using G = TileGeom<DIM, TR, TC>;
    using L = SmemLayout<DIM, TR, TC, NSTAGE>;
    StencilVariant v;
    v.dim = DIM;
    v.epi = EPI;
    v.exact = EXACT ? 1 : 0;
    v.tr = TR;
    v.tc = (DIM == 3) ? TC : 1;
    v.nt = NT;
    v.nstage = NSTAGE;
    v.smem_bytes = L::total;
    v.box_rows = G::LR;
    v.box_cols = G::LC;
    v.box_cols_bc = G::LC_BC;
    v.fn = reinterpret_cast<const void *>(&stencil_iteration_kernel<DIM, TR, TC, NT, NSTAGE, EPI, EXACT>);
    return v;
}

}  // namespace asets
