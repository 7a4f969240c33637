// Per-voxel label updates of the multi-label models, run after the stencil
// kernel has written the new flow divergence of every label.
//
//  Potts:    pt_k = min(ps + u_k/cc - dv_k, Ct_k) with the previous ps
//            (maxflow/asetsPotts3D_mex.c:440-471), then the shared source flow
//            and the multipliers (updatePSU, :474-521).
//  Ishikawa: the sink-flow chain over ordered labels, lowest first, each layer
//            using the just-updated layer below (asetsIshikawa3D_mex.c:498-576),
//            then the multipliers (updateU, :578-610).
//
// Both accumulate erriter and close the iteration (iteration_end.cuh).
// Voxels are visited in the padded layout; each label slice is contiguous in
// rows, so every label access is a coalesced stream.
#include "internal.h"
#include "iteration_end.cuh"

namespace asets {

constexpr int kLabelThreads = 256;

// Walk this warp's 32-element row segments of the padded layout: segment
// (row, seg) covers rows elements seg*32 .. seg*32+31 of padded row `row`
// (label 0); stepping by the number of warps in the grid needs no division
// inside the loop.
struct SegWalk {
    unsigned int row, seg, drow, dseg, cpr;
    __device__ SegWalk(int nr)
    {
        const unsigned int warps = gridDim.x * (kLabelThreads / 32);
        const unsigned int wid = blockIdx.x * (kLabelThreads / 32) + (threadIdx.x >> 5);
        cpr = (unsigned int)(nr + 31) >> 5;
        row = wid / cpr;
        seg = wid % cpr;
        drow = warps / cpr;
        dseg = warps % cpr;
    }
    __device__ void next()
    {
        row += drow;
        seg += dseg;
        if (seg >= cpr) {
            seg -= cpr;
            ++row;
        }
    }
};

// u/cc: IEEE division as the reference (EXACT), or times 1/cc (fast).
template <bool EXACT>
__device__ __forceinline__ float over_cc(float u, float cc, float inv_cc)
{
    return EXACT ? __fdiv_rn(u, cc) : u * inv_cc;
}

// LFIX > 0: label count known at compile time (register arrays);
// LFIX == 0: any label count, second pass re-reads dv_k and the new pt_k
// (same operands, so the same bits).
template <int LFIX, bool EXACT>
__global__ void __launch_bounds__(kLabelThreads) potts_label_kernel(LabelArgs A)
{
    __shared__ double s_red[kLabelThreads / 32];
    __shared__ int s_is_last;
    IterControl *ctl = A.ctl;
    if (*(volatile int *)&ctl->done)
        return;
    const int it = *(volatile int *)&ctl->iter;
    const int L = LFIX > 0 ? LFIX : A.nlab;
    const float cc = A.cc, inv_cc = A.inv_cc;
    const float inv_l = 1.0f / (float)L;
    const unsigned int S = (unsigned int)A.label_stride;
    const int lane = threadIdx.x & 31;
    float erru = 0.0f;
    for (SegWalk w(A.nr); w.row < A.rows; w.next()) {
        const int r = (int)(w.seg << 5) + lane;
        if (r >= A.nr)
            continue;
        const unsigned int g = w.row * (unsigned int)A.pitch + (unsigned int)r;
        const float ps = A.ps[g];
        float fsum = 0.0f;
        if constexpr (LFIX > 0) {
            float ft[LFIX], uu[LFIX];
#pragma unroll
            for (int k = 0; k < LFIX; ++k) {
                const unsigned int o = g + k * S;
                const float u = A.u[o];
                const float uc = over_cc<EXACT>(u, cc, inv_cc);
                const float dv = A.dv[o];
                const float ctv = A.ct[o];
                float pt = (ps + uc) - dv;
                pt = (pt < ctv) ? pt : ctv;
                A.pt[o] = pt;
                ft[k] = dv + pt;
                uu[k] = u;
                fsum += (ft[k] - uc);
            }
            const float ps_n = (EXACT ? __fdiv_rn(fsum, (float)L) : fsum * inv_l) + A.inv_cc_l;
            A.ps[g] = ps_n;
#pragma unroll
            for (int k = 0; k < LFIX; ++k) {
                const float e = cc * (ft[k] - ps_n);
                A.u[g + k * S] = uu[k] - e;
                erru += abs_ref(e);
            }
        } else {
            for (int k = 0; k < L; ++k) {
                const unsigned int o = g + k * S;
                const float uc = over_cc<EXACT>(A.u[o], cc, inv_cc);
                const float dv = A.dv[o];
                const float ctv = A.ct[o];
                float pt = (ps + uc) - dv;
                pt = (pt < ctv) ? pt : ctv;
                A.pt[o] = pt;
                fsum += ((dv + pt) - uc);
            }
            const float ps_n = (EXACT ? __fdiv_rn(fsum, (float)L) : fsum * inv_l) + A.inv_cc_l;
            A.ps[g] = ps_n;
            for (int k = 0; k < L; ++k) {
                const unsigned int o = g + k * S;
                const float e = cc * ((A.dv[o] + A.pt[o]) - ps_n);
                A.u[o] = A.u[o] - e;
                erru += abs_ref(e);
            }
        }
    }
    finish_iteration<kLabelThreads>(erru, ctl, A.partials, A.cvg, it, s_red, &s_is_last, A.done_count);
}

template <bool EXACT>
__global__ void __launch_bounds__(kLabelThreads) ishikawa_label_kernel(LabelArgs A)
{
    __shared__ double s_red[kLabelThreads / 32];
    __shared__ int s_is_last;
    IterControl *ctl = A.ctl;
    if (*(volatile int *)&ctl->done)
        return;
    const int it = *(volatile int *)&ctl->iter;
    const int L = A.nlab;
    const float cc = A.cc, inv_cc = A.inv_cc;
    const unsigned int S = (unsigned int)A.label_stride;
    const int lane = threadIdx.x & 31;
    float erru = 0.0f;
    for (SegWalk w(A.nr); w.row < A.rows; w.next()) {
        const int r = (int)(w.seg << 5) + lane;
        if (r >= A.nr)
            continue;
        const unsigned int g = w.row * (unsigned int)A.pitch + (unsigned int)r;
        // layer below k: new pt, its divergence and multiplier
        float pt_below = 0.f, dv_below = 0.f, ucc_below = 0.f, u_below = 0.f;
        for (int k = 0; k < L; ++k) {
            const unsigned int o = g + k * S;
            float dv_k = 0.f, u_k = 0.f, ucc_k = 0.f, pt_up = 0.f;
            if (k < L - 1) {
                dv_k = A.dv[o];
                u_k = A.u[o];
                ucc_k = over_cc<EXACT>(u_k, cc, inv_cc);
                pt_up = A.pt[o + S];  // previous pt_{k+1}
            }
            float fpt;
            if (k == 0) {
                fpt = ((dv_k + pt_up) - ucc_k) + inv_cc;
            } else if (k < L - 1) {
                fpt = ((-dv_below) + pt_below) + ucc_below;
                fpt = fpt + ((dv_k + pt_up) - ucc_k);
                fpt = fpt * 0.5f;  // = fpt / 2 exactly
            } else {
                fpt = ((-dv_below) + pt_below) + ucc_below;
            }
            const float pt_new = min_ref(fpt, A.ct[o]);
            A.pt[o] = pt_new;
            if (k >= 1) {
                // multiplier of layer k-1: cc*(dv + pt_{k} - pt_{k-1}), new pts
                const float e = cc * ((dv_below + pt_new) - pt_below);
                A.u[o - S] = u_below - e;
                erru += abs_ref(e);
            }
            pt_below = pt_new;
            dv_below = dv_k;
            ucc_below = ucc_k;
            u_below = u_k;
        }
    }
    finish_iteration<kLabelThreads>(erru, ctl, A.partials, A.cvg, it, s_red, &s_is_last, A.done_count);
}

int label_kernel_grid(long long cells, int num_sms)
{
    long long blocks = (cells + kLabelThreads - 1) / kLabelThreads;
    long long cap = (long long)num_sms * 4;  // all resident (<= 64 registers per thread)
    if (blocks < 1)
        blocks = 1;
    return (int)(blocks < cap ? blocks : cap);
}

template <bool EXACT>
static void potts_launch(const LabelArgs &a, int grid, cudaStream_t st)
{
    switch (a.nlab) {
    case 2: potts_label_kernel<2, EXACT><<<grid, kLabelThreads, 0, st>>>(a); break;
    case 3: potts_label_kernel<3, EXACT><<<grid, kLabelThreads, 0, st>>>(a); break;
    case 4: potts_label_kernel<4, EXACT><<<grid, kLabelThreads, 0, st>>>(a); break;
    case 5: potts_label_kernel<5, EXACT><<<grid, kLabelThreads, 0, st>>>(a); break;
    case 6: potts_label_kernel<6, EXACT><<<grid, kLabelThreads, 0, st>>>(a); break;
    case 8: potts_label_kernel<8, EXACT><<<grid, kLabelThreads, 0, st>>>(a); break;
    default: potts_label_kernel<0, EXACT><<<grid, kLabelThreads, 0, st>>>(a); break;
    }
}

cudaError_t launch_potts_labels(const LabelArgs &a, int grid, cudaStream_t st)
{
    if (a.exact)
        potts_launch<true>(a, grid, st);
    else
        potts_launch<false>(a, grid, st);
    return cudaGetLastError();
}

cudaError_t launch_ishikawa_labels(const LabelArgs &a, int grid, cudaStream_t st)
{
    if (a.exact)
        ishikawa_label_kernel<true><<<grid, kLabelThreads, 0, st>>>(a);
    else
        ishikawa_label_kernel<false><<<grid, kLabelThreads, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace asets
