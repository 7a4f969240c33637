// Grid transfer of the multilevel (coarse-to-fine) solve: restriction of the
// inputs to a grid with half the cells per axis, and prolongation of a solved
// coarse state to the fine grid as its initial state.
//
// Both work on the solver's padded layout (kernel view rows r = Matlab y,
// columns c = Matlab x in 3D, stream s = z in 3D / x in 2D).  A coarse cell
// covers the fine cells 2i and 2i+1 of each axis that has more than one cell
// (one cell at an odd border).
//
// Restriction: a coarse cell with a 2x2x2 block of the fine grid has 8 times
// the data term and its faces 4 times the fine faces' total variation, so
// the coarse problem of the same energy (divided by 4) has cost terms
// 2*mean(C) and the same alpha (mean over the block); 2D gives the same
// factors (4 cells, 2 faces).
// Prolongation: u copied to the covered fine cells; ps, pt halved (they are
// bounded by the cost terms); flows (bounded by alpha) copied in the
// transverse axes, and along their own axis taken from the coarse face at
// even fine faces and averaged from the two neighbouring coarse faces at odd
// ones (the face between the two fine cells of one coarse cell), with zero
// beyond the last coarse face.
#include "internal.h"

namespace asets {

__global__ void restrict_kernel(const GridXfer X, const float *__restrict__ src,
                                float *__restrict__ dst, int labels, float scale)
{
    const long long per_label = (long long)X.c.nr * X.c.nc * X.c.ns;
    const long long total = per_label * labels;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(i % X.c.nr);
        const long long q = i / X.c.nr;
        const int c = (int)(q % X.c.nc);
        const long long q2 = q / X.c.nc;
        const int s = (int)(q2 % X.c.ns);
        const int l = (int)(q2 / X.c.ns);
        const int r1 = min(2 * r + 1, X.f.nr - 1) - 2 * r;
        const int c1 = X.f.nc > 1 ? min(2 * c + 1, X.f.nc - 1) - 2 * c : 0;
        const int s1 = X.f.ns > 1 ? min(2 * s + 1, X.f.ns - 1) - 2 * s : 0;
        const float *f = src + (long long)l * X.f.cells;
        float sum = 0.f;
        int cnt = 0;
        for (int ds = 0; ds <= s1; ++ds)
            for (int dc = 0; dc <= c1; ++dc)
                for (int dr = 0; dr <= r1; ++dr) {
                    const int fs = (X.f.ns > 1 ? 2 * s : s) + ds;
                    const int fc = (X.f.nc > 1 ? 2 * c : c) + dc;
                    sum = __fadd_rn(sum, f[(long long)fs * X.f.plane + (long long)fc * X.f.pitch + 2 * r + dr]);
                    ++cnt;
                }
        dst[(long long)l * X.c.cells + (long long)s * X.c.plane + (long long)c * X.c.pitch + r] =
            __fmul_rn(__fdiv_rn(sum, (float)cnt), scale);
    }
}

// axis: -1 = a cell quantity (copied, times scale); 0 = flow along rows,
// 1 = along columns, 2 = along the stream axis.
__global__ void prolong_kernel(const GridXfer X, const float *__restrict__ src,
                               float *__restrict__ dst, int labels, float scale, int axis)
{
    const long long per_label = (long long)X.f.nr * X.f.nc * X.f.ns;
    const long long total = per_label * labels;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(i % X.f.nr);
        const long long q = i / X.f.nr;
        const int c = (int)(q % X.f.nc);
        const long long q2 = q / X.f.nc;
        const int s = (int)(q2 % X.f.ns);
        const int l = (int)(q2 / X.f.ns);
        int cr = r >> 1;
        int cc = X.f.nc > 1 ? c >> 1 : c;
        int cs = X.f.ns > 1 ? s >> 1 : s;
        const float *g = src + (long long)l * X.c.cells;
        auto at = [&](int rr, int c2, int s2) -> float {
            if (rr >= X.c.nr || c2 >= X.c.nc || s2 >= X.c.ns)
                return 0.f;  // beyond the last coarse face
            return g[(long long)s2 * X.c.plane + (long long)c2 * X.c.pitch + rr];
        };
        float v;
        const int fi = axis == 0 ? r : (axis == 1 ? c : s);
        const bool split = axis >= 0 && (axis == 0 || (axis == 1 ? X.f.nc > 1 : X.f.ns > 1));
        if (split && (fi & 1)) {
            const float a = at(cr, cc, cs);
            const float b = at(cr + (axis == 0), cc + (axis == 1), cs + (axis == 2));
            v = __fmul_rn(__fadd_rn(a, b), 0.5f);
        } else {
            v = at(cr, cc, cs);
        }
        dst[(long long)l * X.f.cells + (long long)s * X.f.plane + (long long)c * X.f.pitch + r] =
            __fmul_rn(v, scale);
    }
}

static int xfer_grid(long long n, int num_sms)
{
    long long b = (n + 255) / 256;
    const long long cap = (long long)num_sms * 16;
    return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

cudaError_t launch_restrict(const GridXfer &X, const float *src, float *dst, int labels,
                            float scale, int num_sms, cudaStream_t st)
{
    const long long n = (long long)X.c.nr * X.c.nc * X.c.ns * labels;
    restrict_kernel<<<xfer_grid(n, num_sms), 256, 0, st>>>(X, src, dst, labels, scale);
    return cudaGetLastError();
}

cudaError_t launch_prolong(const GridXfer &X, const float *src, float *dst, int labels,
                           float scale, int axis, int num_sms, cudaStream_t st)
{
    const long long n = (long long)X.f.nr * X.f.nc * X.f.ns * labels;
    prolong_kernel<<<xfer_grid(n, num_sms), 256, 0, st>>>(X, src, dst, labels, scale, axis);
    return cudaGetLastError();
}

}  // namespace asets
