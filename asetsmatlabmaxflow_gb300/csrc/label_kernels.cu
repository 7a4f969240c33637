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
    __device__ SegWalk(int nr, int width = 32)
    {
        const unsigned int warps = gridDim.x * (kLabelThreads / 32);
        const unsigned int wid = blockIdx.x * (kLabelThreads / 32) + (threadIdx.x >> 5);
        cpr = (unsigned int)(nr + width - 1) / (unsigned int)width;
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

// VEC adjacent voxels of one row per thread, as one 8- or 16-byte access
// (n < VEC: the row's last voxels, element by element; the rest read as 0
// and are not stored).
template <int VEC>
__device__ __forceinline__ void ld_vec(const float *p, float (&v)[VEC], int n)
{
    if (n == VEC) {
        if constexpr (VEC == 4) {
            const float4 t = *reinterpret_cast<const float4 *>(p);
            v[0] = t.x;
            v[1] = t.y;
            v[2] = t.z;
            v[3] = t.w;
        } else if constexpr (VEC == 2) {
            const float2 t = *reinterpret_cast<const float2 *>(p);
            v[0] = t.x;
            v[1] = t.y;
        } else {
            v[0] = p[0];
        }
    } else {
#pragma unroll
        for (int i = 0; i < VEC; ++i)
            v[i] = (i < n) ? p[i] : 0.f;
    }
}
template <int VEC>
__device__ __forceinline__ void st_vec(float *p, const float (&v)[VEC], int n)
{
    if (n == VEC) {
        if constexpr (VEC == 4)
            *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
        else if constexpr (VEC == 2)
            *reinterpret_cast<float2 *>(p) = make_float2(v[0], v[1]);
        else
            p[0] = v[0];
    } else {
#pragma unroll
        for (int i = 0; i < VEC; ++i)
            if (i < n)
                p[i] = v[i];
    }
}

// The Potts update for a known label count with VEC voxels per thread:
// the same per-voxel operations as potts_label_kernel (so the same u bits),
// wider accesses and fewer instructions per voxel.  Rows are padded to a
// multiple of 4 floats and label slices are whole padded volumes, so every
// full group is 4*VEC-byte aligned.
template <int LFIX, bool EXACT, int VEC>
__global__ void __launch_bounds__(kLabelThreads) potts_label_kernel_v(LabelArgs A)
{
    __shared__ double s_red[kLabelThreads / 32];
    __shared__ int s_is_last;
    IterControl *ctl = A.ctl;
    if (*(volatile int *)&ctl->done)
        return;
    const int it = *(volatile int *)&ctl->iter;
    const float cc = A.cc, inv_cc = A.inv_cc;
    const float inv_l = 1.0f / (float)LFIX;
    const unsigned int S = (unsigned int)A.label_stride;
    const int lane = threadIdx.x & 31;
    float erru = 0.0f;
    for (SegWalk w(A.nr, 32 * VEC); w.row < A.rows; w.next()) {
        const int r = (int)(w.seg * (32 * VEC)) + lane * VEC;
        if (r >= A.nr)
            continue;
        const int n = min(VEC, A.nr - r);
        const unsigned int g = w.row * (unsigned int)A.pitch + (unsigned int)r;
        float ps[VEC], fsum[VEC];
        float ft[LFIX][VEC], uu[LFIX][VEC];
        ld_vec<VEC>(A.ps + g, ps, n);
#pragma unroll
        for (int i = 0; i < VEC; ++i)
            fsum[i] = 0.0f;
#pragma unroll
        for (int k = 0; k < LFIX; ++k) {
            const unsigned int o = g + k * S;
            float u[VEC], dv[VEC], ctv[VEC], pt[VEC];
            ld_vec<VEC>(A.u + o, u, n);
            ld_vec<VEC>(A.dv + o, dv, n);
            ld_vec<VEC>(A.ct + o, ctv, n);
#pragma unroll
            for (int i = 0; i < VEC; ++i) {
                const float uc = over_cc<EXACT>(u[i], cc, inv_cc);
                float p = (ps[i] + uc) - dv[i];
                p = (p < ctv[i]) ? p : ctv[i];
                pt[i] = p;
                ft[k][i] = dv[i] + p;
                uu[k][i] = u[i];
                fsum[i] += (ft[k][i] - uc);
            }
            st_vec<VEC>(A.pt + o, pt, n);
        }
        float ps_n[VEC];
#pragma unroll
        for (int i = 0; i < VEC; ++i)
            ps_n[i] = (EXACT ? __fdiv_rn(fsum[i], (float)LFIX) : fsum[i] * inv_l) + A.inv_cc_l;
        st_vec<VEC>(A.ps + g, ps_n, n);
#pragma unroll
        for (int k = 0; k < LFIX; ++k) {
            float un[VEC];
#pragma unroll
            for (int i = 0; i < VEC; ++i) {
                const float e = cc * (ft[k][i] - ps_n[i]);
                un[i] = uu[k][i] - e;
                if (i < n)
                    erru += abs_ref(e);
            }
            st_vec<VEC>(A.u + g + k * S, un, n);
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

// The Ishikawa update with VEC voxels per thread: the same per-voxel chain
// as ishikawa_label_kernel (so the same u bits), wider accesses.
template <bool EXACT, int VEC>
__global__ void __launch_bounds__(kLabelThreads) ishikawa_label_kernel_v(LabelArgs A)
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
    for (SegWalk w(A.nr, 32 * VEC); w.row < A.rows; w.next()) {
        const int r = (int)(w.seg * (32 * VEC)) + lane * VEC;
        if (r >= A.nr)
            continue;
        const int n = min(VEC, A.nr - r);
        const unsigned int g = w.row * (unsigned int)A.pitch + (unsigned int)r;
        // layer below k: new pt, its divergence and multiplier
        float pt_below[VEC], dv_below[VEC], ucc_below[VEC], u_below[VEC];
#pragma unroll
        for (int i = 0; i < VEC; ++i)
            pt_below[i] = dv_below[i] = ucc_below[i] = u_below[i] = 0.f;
        for (int k = 0; k < L; ++k) {
            const unsigned int o = g + k * S;
            float dv_k[VEC], u_k[VEC], ucc_k[VEC], pt_up[VEC], ctv[VEC], pt_new[VEC];
            if (k < L - 1) {
                ld_vec<VEC>(A.dv + o, dv_k, n);
                ld_vec<VEC>(A.u + o, u_k, n);
                ld_vec<VEC>(A.pt + o + S, pt_up, n);  // previous pt_{k+1}
            } else {
#pragma unroll
                for (int i = 0; i < VEC; ++i)
                    dv_k[i] = u_k[i] = pt_up[i] = 0.f;
            }
            ld_vec<VEC>(A.ct + o, ctv, n);
#pragma unroll
            for (int i = 0; i < VEC; ++i) {
                ucc_k[i] = (k < L - 1) ? over_cc<EXACT>(u_k[i], cc, inv_cc) : 0.f;
                float fpt;
                if (k == 0) {
                    fpt = ((dv_k[i] + pt_up[i]) - ucc_k[i]) + inv_cc;
                } else if (k < L - 1) {
                    fpt = ((-dv_below[i]) + pt_below[i]) + ucc_below[i];
                    fpt = fpt + ((dv_k[i] + pt_up[i]) - ucc_k[i]);
                    fpt = fpt * 0.5f;  // = fpt / 2 exactly
                } else {
                    fpt = ((-dv_below[i]) + pt_below[i]) + ucc_below[i];
                }
                pt_new[i] = min_ref(fpt, ctv[i]);
            }
            st_vec<VEC>(A.pt + o, pt_new, n);
            if (k >= 1) {
                // multiplier of layer k-1: cc*(dv + pt_{k} - pt_{k-1}), new pts
                float un[VEC];
#pragma unroll
                for (int i = 0; i < VEC; ++i) {
                    const float e = cc * ((dv_below[i] + pt_new[i]) - pt_below[i]);
                    un[i] = u_below[i] - e;
                    if (i < n)
                        erru += abs_ref(e);
                }
                st_vec<VEC>(A.u + o - S, un, n);
            }
#pragma unroll
            for (int i = 0; i < VEC; ++i) {
                pt_below[i] = pt_new[i];
                dv_below[i] = dv_k[i];
                ucc_below[i] = ucc_k[i];
                u_below[i] = u_k[i];
            }
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

template <int L, bool EXACT>
static void potts_launch_l(const LabelArgs &a, int grid, cudaStream_t st, int vec)
{
    if (vec == 2)
        potts_label_kernel_v<L, EXACT, 2><<<grid, kLabelThreads, 0, st>>>(a);
    else
        potts_label_kernel<L, EXACT><<<grid, kLabelThreads, 0, st>>>(a);
}

// voxels per thread: 2 on rows of 64 and more (a short row would leave
// lanes of the 64-element segment idle), else 1.  Four per thread measured
// slower: at 80 registers four 256-thread blocks no longer fit on an SM.
static int potts_vec(int nr) { return nr >= 64 ? 2 : 1; }

template <bool EXACT>
static void potts_launch(const LabelArgs &a, int grid, cudaStream_t st)
{
    const int vec = potts_vec(a.nr);
    switch (a.nlab) {
    case 2: potts_launch_l<2, EXACT>(a, grid, st, vec); break;
    case 3: potts_launch_l<3, EXACT>(a, grid, st, vec); break;
    case 4: potts_launch_l<4, EXACT>(a, grid, st, vec); break;
    case 5: potts_launch_l<5, EXACT>(a, grid, st, vec); break;
    case 6: potts_launch_l<6, EXACT>(a, grid, st, vec); break;
    case 8: potts_launch_l<8, EXACT>(a, grid, st, vec); break;
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
    const bool two = potts_vec(a.nr) == 2;  // the same rule: two voxels on rows of 64+
    if (a.exact) {
        if (two)
            ishikawa_label_kernel_v<true, 2><<<grid, kLabelThreads, 0, st>>>(a);
        else
            ishikawa_label_kernel<true><<<grid, kLabelThreads, 0, st>>>(a);
    } else {
        if (two)
            ishikawa_label_kernel_v<false, 2><<<grid, kLabelThreads, 0, st>>>(a);
        else
            ishikawa_label_kernel<false><<<grid, kLabelThreads, 0, st>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace asets
