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

// LFIX > 0: label count known at compile time (register arrays);
// LFIX == 0: any label count, second pass re-reads dv_k and the new pt_k
// (same operands, so the same bits).
template <int LFIX>
__global__ void __launch_bounds__(kLabelThreads) potts_label_kernel(LabelArgs A)
{
    __shared__ double s_red[kLabelThreads / 32];
    __shared__ int s_is_last;
    IterControl *ctl = A.ctl;
    if (*(volatile int *)&ctl->done)
        return;
    const int it = *(volatile int *)&ctl->iter;
    const int L = LFIX > 0 ? LFIX : A.nlab;
    const float cc = A.cc;
    const long long S = A.label_stride;
    float erru = 0.0f;
    for (long long g = blockIdx.x * (long long)kLabelThreads + threadIdx.x; g < A.cells;
         g += (long long)gridDim.x * kLabelThreads) {
        if ((int)(g % A.pitch) >= A.nr)
            continue;
        const float ps = A.ps[g];
        float fsum = 0.0f;
        if constexpr (LFIX > 0) {
            float ft[LFIX], uu[LFIX];
#pragma unroll
            for (int k = 0; k < LFIX; ++k) {
                const long long o = g + k * S;
                const float u = A.u[o];
                const float uc = __fdiv_rn(u, cc);
                const float dv = A.dv[o];
                const float ctv = A.ct[o];
                float pt = (ps + uc) - dv;
                pt = (pt < ctv) ? pt : ctv;
                A.pt[o] = pt;
                ft[k] = dv + pt;
                uu[k] = u;
                fsum += (ft[k] - uc);
            }
            const float ps_n = __fdiv_rn(fsum, (float)L) + A.inv_cc_l;
            A.ps[g] = ps_n;
#pragma unroll
            for (int k = 0; k < LFIX; ++k) {
                const float e = cc * (ft[k] - ps_n);
                A.u[g + k * S] = uu[k] - e;
                erru += abs_ref(e);
            }
        } else {
            for (int k = 0; k < L; ++k) {
                const long long o = g + k * S;
                const float uc = __fdiv_rn(A.u[o], cc);
                const float dv = A.dv[o];
                const float ctv = A.ct[o];
                float pt = (ps + uc) - dv;
                pt = (pt < ctv) ? pt : ctv;
                A.pt[o] = pt;
                fsum += ((dv + pt) - uc);
            }
            const float ps_n = __fdiv_rn(fsum, (float)L) + A.inv_cc_l;
            A.ps[g] = ps_n;
            for (int k = 0; k < L; ++k) {
                const long long o = g + k * S;
                const float e = cc * ((A.dv[o] + A.pt[o]) - ps_n);
                A.u[o] = A.u[o] - e;
                erru += abs_ref(e);
            }
        }
    }
    finish_iteration<kLabelThreads>(erru, ctl, A.partials, A.cvg, it, s_red, &s_is_last);
}

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
    const long long S = A.label_stride;
    float erru = 0.0f;
    for (long long g = blockIdx.x * (long long)kLabelThreads + threadIdx.x; g < A.cells;
         g += (long long)gridDim.x * kLabelThreads) {
        if ((int)(g % A.pitch) >= A.nr)
            continue;
        // layer below k: new pt, its divergence and multiplier
        float pt_below = 0.f, dv_below = 0.f, ucc_below = 0.f, u_below = 0.f;
        for (int k = 0; k < L; ++k) {
            const long long o = g + k * S;
            float dv_k = 0.f, u_k = 0.f, ucc_k = 0.f, pt_up = 0.f;
            if (k < L - 1) {
                dv_k = A.dv[o];
                u_k = A.u[o];
                ucc_k = __fdiv_rn(u_k, cc);
                pt_up = A.pt[o + S];  // previous pt_{k+1}
            }
            float fpt;
            if (k == 0) {
                fpt = ((dv_k + pt_up) - ucc_k) + inv_cc;
            } else if (k < L - 1) {
                fpt = ((-dv_below) + pt_below) + ucc_below;
                fpt = fpt + ((dv_k + pt_up) - ucc_k);
                fpt = fpt / 2.0f;
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
    finish_iteration<kLabelThreads>(erru, ctl, A.partials, A.cvg, it, s_red, &s_is_last);
}

int label_kernel_grid(long long cells, int num_sms)
{
    long long blocks = (cells + kLabelThreads - 1) / kLabelThreads;
    long long cap = (long long)num_sms * 8;
    if (blocks < 1)
        blocks = 1;
    return (int)(blocks < cap ? blocks : cap);
}

cudaError_t launch_potts_labels(const LabelArgs &a, int grid, cudaStream_t st)
{
    switch (a.nlab) {
    case 2: potts_label_kernel<2><<<grid, kLabelThreads, 0, st>>>(a); break;
    case 3: potts_label_kernel<3><<<grid, kLabelThreads, 0, st>>>(a); break;
    case 4: potts_label_kernel<4><<<grid, kLabelThreads, 0, st>>>(a); break;
    case 5: potts_label_kernel<5><<<grid, kLabelThreads, 0, st>>>(a); break;
    case 6: potts_label_kernel<6><<<grid, kLabelThreads, 0, st>>>(a); break;
    case 8: potts_label_kernel<8><<<grid, kLabelThreads, 0, st>>>(a); break;
    default: potts_label_kernel<0><<<grid, kLabelThreads, 0, st>>>(a); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_ishikawa_labels(const LabelArgs &a, int grid, cudaStream_t st)
{
    ishikawa_label_kernel<<<grid, kLabelThreads, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace asets
