// Multi-label 2D iteration (Potts, Ishikawa) on 16 x 16 tiles, for small
// images: the square-tile scheme of stencil2d_tile.cuh with every label of
// the tile in one block.
//
// A block loads the old state of its tile and two-cell halo for all labels
// at once (16-byte cp.async copies through L2, zero-filled outside the
// image: the zero-flux border), then per flow label runs the phases of the
// binary tile kernel -- gk, b', g2, b'' (stored), the divergence on the tile
// -- in groups of 128 threads, one label per group at a time, each group
// ordered by its own named barrier -- and finally the per-pixel label update
// over all labels: Potts pt_k,
// the source flow ps (terms summed in label order) and the multipliers
// (maxflow/asetsPotts2D_mex.c:365-434); Ishikawa the ordered sink-flow chain
// and the multipliers (maxflow/asetsIshikawa2D_mex.c:392-482).  The label
// count is a run-time value (ProblemDesc::nlab_items flow labels); the
// shared memory of a launch is sized for its label count
// (LTileGeom::smem_bytes).  Every value is the two-pass form's
// float expression in the same order: EXACT results are bit-identical.
// Like the binary tile kernel it runs one launch per iteration or the whole
// solve in one cooperative launch (every block resident, one or more tiles
// each, a grid barrier between iterations); new pt, u and ps go to the
// other parity.
#pragma once

#include "stencil2d_tile.cuh"

namespace asets {

template <int MODEL>
struct LTileGeom {
    static_assert(MODEL == 1 || MODEL == 2, "Potts (1) or Ishikawa (2)");
    static constexpr int R = 16, S = 16;      // tile rows, stream columns
    static constexpr int FR = 24;             // frame rows r0-4 .. r0+19: 16-byte chunks
    static constexpr int RO = 2;              // frame row of pixel row r0-2
    static constexpr int FC = S + 5;          // frame columns s0-2 .. s0+S+2
    static constexpr int F = FR * FC;         // floats per frame (a multiple of 4)
    static constexpr int GROUPS = 4;          // label groups of 128 threads (group_sync)
    static constexpr int NT = 128 * GROUPS;
    static constexpr int FLMAX = 8;           // flow labels
    static constexpr int LMAX = (MODEL == 1) ? 8 : 9;
    // frames: BR, BS, U, AL per flow label, PT per label, PS (Potts), then
    // GK, BR1, BS1, G2 per group; then DV per flow label and CT per label on
    // the tile
    static constexpr int frames(int fl, int l) { return 4 * fl + l + (MODEL == 1 ? 1 : 0) + 4 * GROUPS; }
    // shared memory of a launch for fl flow labels and l labels: a base and
    // a share per flow label and per label (the runtime sizes launches so)
    static constexpr int smem_base() { return ((MODEL == 1 ? 1 : 0) + 4 * GROUPS) * F * 4 + 16; }
    static constexpr int smem_per_fl() { return (4 * F + R * S) * 4; }
    static constexpr int smem_per_l() { return (F + R * S) * 4; }
    static constexpr int smem_bytes(int fl, int l)
    {
        return smem_base() + fl * smem_per_fl() + l * smem_per_l();
    }
};

// barrier of one 128-thread label group (ids 1..4; 0 is __syncthreads).
// Immediate ids: a register id would reserve all sixteen barriers.
__device__ __forceinline__ void group_sync(int g)
{
    switch (g) {
    case 0: asm volatile("bar.sync 1, 128;" ::: "memory"); break;
    case 1: asm volatile("bar.sync 2, 128;" ::: "memory"); break;
    case 2: asm volatile("bar.sync 3, 128;" ::: "memory"); break;
    default: asm volatile("bar.sync 4, 128;" ::: "memory"); break;
    }
}

// 16-byte asynchronous copy global -> shared through L2; `bytes` < 16
// zero-fills the rest (0: the whole chunk)
__device__ __forceinline__ void cp_async16(float *dst, const float *src, int bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(dst)), "l"(src),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

template <int MODEL, int NT, bool EXACT>
__device__ __forceinline__ float ltile_iteration(const ProblemDesc &P, int par, int li, float *sm)
{
    using G = LTileGeom<MODEL>;
    constexpr int R = G::R, S = G::S, FR = G::FR, RO = G::RO, FC = G::FC, F = G::F;
    const int tid = threadIdx.x;
    const int FL = P.nlab_items;
    const int L = (MODEL == 1) ? FL : FL + 1;
    const int nr = P.nr, ns = P.ns;
    const float cc = P.cc, inv_cc = P.inv_cc, steps = P.steps;
    const int r0 = (li % P.tiles_r) * R;
    const int s0 = (li / P.tiles_r) * S;
    const unsigned int pitch = (unsigned int)P.plane_stride;
    const unsigned int lst = (unsigned int)P.label_stride;
    float *BRf = sm, *BSf = BRf + FL * F, *Uf = BSf + FL * F, *ALf = Uf + FL * F;
    float *PTf = ALf + FL * F;
    float *PSf = PTf + L * F;                                   // Potts only
    float *Wk = PSf + (MODEL == 1 ? F : 0);                     // per group: GK, BR1, BS1, G2
    float *DV = Wk + 4 * G::GROUPS * F, *CT = DV + FL * R * S;
    // old state (the other parity), and the new
    const float *src_br = P.dst_b[par ^ 1][SL_BR], *src_bs = P.dst_b[par ^ 1][SL_BS];
    const float *src_u = P.dst_s[par ^ 1][2];
    const float *src_pt = (MODEL == 1) ? P.dst_s[par ^ 1][1] : P.dst_s[par ^ 1][0];
    const float *src_ps = P.dst_s[par ^ 1][0];                  // Potts
    float *d_br = P.dst_b[par][SL_BR], *d_bs = P.dst_b[par][SL_BS];
    float *d_u = P.dst_s[par][2];
    float *d_pt = (MODEL == 1) ? P.dst_s[par][1] : P.dst_s[par][0];
    float *d_ps = P.dst_s[par][0];                              // Potts

    // ---- all loads in flight at once: frame chunk (column c, rows
    // r0-4+4j .. +3) of each frame array, Ct on the tile
    {
        const int nframe = 4 * FL + L + (MODEL == 1 ? 1 : 0);
        const int chunks = FC * (FR / 4);
        for (int i = tid; i < nframe * chunks; i += NT) {
            const int fr = i / chunks, rem = i - fr * chunks;
            const int c = rem / (FR / 4), j = rem - c * (FR / 4);
            const int r = r0 - 4 + 4 * j, s = s0 - 2 + c;
            const float *src;
            int lab;
            if (fr < FL) { src = src_br; lab = fr; }
            else if (fr < 2 * FL) { src = src_bs; lab = fr - FL; }
            else if (fr < 3 * FL) { src = src_u; lab = fr - 2 * FL; }
            else if (fr < 4 * FL) { src = P.alpha; lab = fr - 3 * FL; }
            else if (fr < 4 * FL + L) { src = src_pt; lab = fr - 4 * FL; }
            else { src = src_ps; lab = 0; }
            int bytes = 0;
            if (s >= 0 && s < ns && r >= 0 && r < nr)
                bytes = min(16, (nr - r) * 4);
            const float *g = bytes ? src + (unsigned int)lab * lst + (unsigned int)s * pitch + r : src;
            cp_async16(sm + fr * F + c * FR + 4 * j, g, bytes);
        }
        // Ct of the tile: L labels x S columns x R/4 chunks
        for (int i = tid; i < L * S * (R / 4); i += NT) {
            const int l = i / (S * (R / 4)), rem = i - l * (S * (R / 4));
            const int c = rem / (R / 4), j = rem - c * (R / 4);
            const int r = r0 + 4 * j, s = s0 + c;
            int bytes = 0;
            if (s < ns && r < nr)
                bytes = min(16, (nr - r) * 4);
            const float *g =
                bytes ? P.ct + (unsigned int)l * lst + (unsigned int)s * pitch + r : P.ct;
            cp_async16(CT + l * R * S + c * R + 4 * j, g, bytes);
        }
        cp_async_wait_all();
        __syncthreads();
    }

    // ---- per flow label: gk, b', g2, b'' (stored), the divergence on the
    // tile; group gi takes labels gi, gi + GROUPS, ... with its own work
    // frames and barrier
    static_assert(NT == G::NT, "four label groups of 128 threads");
    const int gi = tid >> 7, gt = tid & 127;
    float *GK = Wk + gi * 4 * F, *BR1 = GK + F, *BS1 = BR1 + F, *G2 = BS1 + F;
    for (int k = gi; k < FL; k += G::GROUPS) {
        float *BR = BRf + k * F, *BS = BSf + k * F;
        const float *U = Uf + k * F, *AL = ALf + k * F;
        const float *S0 = (MODEL == 1) ? PSf : PTf + k * F;         // ps, or pt_k
        const float *S1 = (MODEL == 1) ? PTf + k * F : PTf + (k + 1) * F;  // pt_k, or pt_{k+1}
        for (int i = gt; i < (R + 4) * (S + 4); i += 128) {
            const int c = i / (R + 4), q = i - c * (R + 4);
            const int f = c * FR + RO + q;
            float d = BR[f + 1] - BR[f];
            d = d + BS[f + FR];
            d = d - BS[f];
            GK[f] = d - ((S0[f] - S1[f]) + div_cc<EXACT>(U[f], cc, inv_cc));
        }
        group_sync(gi);
        for (int i = gt; i < (R + 3) * (S + 2); i += 128) {
            const int c = 1 + i / (R + 3), q = 1 + i % (R + 3);
            const int f = c * FR + RO + q;
            const int r = r0 - 2 + q, s = s0 - 2 + c;
            const bool fr_ok = (r >= 1 && r < nr), s_in = (s >= 0 && s < ns);
            BR1[f] = keep_if<EXACT>(steps * (GK[f] - GK[f - 1]) + BR[f], fr_ok && s_in,
                                    fr_ok ? 1.f : 0.f);
        }
        for (int i = gt; i < (R + 2) * (S + 3); i += 128) {
            const int c = 1 + i / (R + 2), q = 1 + i % (R + 2);
            const int f = c * FR + RO + q;
            const int r = r0 - 2 + q, s = s0 - 2 + c;
            const bool inplane = (r >= 0 && r < nr), sb_in = (s >= 1 && s < ns);
            BS1[f] = keep_if<EXACT>(steps * (GK[f] - GK[f - FR]) + BS[f], inplane && sb_in,
                                    sb_in ? 1.f : 0.f);
        }
        group_sync(gi);
        for (int i = gt; i < (R + 2) * (S + 2); i += 128) {
            const int c = 1 + i / (R + 2), q = 1 + i % (R + 2);
            const int f = c * FR + RO + q;
            G2[f] = Proj<EXACT>::gk(BS1[f + FR], BS1[f], BR1[f + 1], BR1[f], AL[f]);
        }
        group_sync(gi);
        const unsigned int lo = (unsigned int)k * lst;
        for (int i = gt; i < (R + 1) * S; i += 128) {
            const int c = 2 + i / (R + 1), q = 2 + i % (R + 1);
            const int f = c * FR + RO + q;
            const int r = r0 - 2 + q, s = s0 - 2 + c;
            const bool fr_ok = (r >= 1 && r < nr), sp_in = (s >= 0 && s < ns);
            const float v = keep_if<EXACT>(((G2[f] + G2[f - 1]) * 0.5f) * BR1[f], fr_ok && sp_in,
                                           fr_ok ? 1.f : 0.f);
            BR[f] = v;
            if (q < R + 2 && r < nr && s < ns)
                d_br[lo + (unsigned int)s * pitch + (unsigned int)r] = v;
        }
        for (int i = gt; i < R * (S + 1); i += 128) {
            const int c = 2 + i / R, q = 2 + i % R;
            const int f = c * FR + RO + q;
            const int r = r0 - 2 + q, s = s0 - 2 + c;
            const bool inplane = (r >= 0 && r < nr), spb_in = (s >= 1 && s < ns);
            const float v = keep_if<EXACT>(((G2[f] + G2[f - FR]) * 0.5f) * BS1[f],
                                           inplane && spb_in, spb_in ? 1.f : 0.f);
            BS[f] = v;
            if (c < S + 2 && r < nr && s < ns)
                d_bs[lo + (unsigned int)s * pitch + (unsigned int)r] = v;
        }
        group_sync(gi);
        for (int i = gt; i < R * S; i += 128) {
            const int c = 2 + i / R, q = 2 + i % R;
            const int f = c * FR + RO + q;
            float dv = BR[f + 1] - BR[f];
            dv = dv + BS[f + FR];
            dv = dv - BS[f];
            DV[k * R * S + i] = dv;
        }
        group_sync(gi);  // the group's work frames are reused by its next label
    }
    __syncthreads();  // every label's divergence

    // ---- the label update of the tile's pixels
    float erru = 0.0f;
    for (int i = tid; i < R * S; i += NT) {
        const int c = i / R, q = i - c * R;
        const int r = r0 + q, s = s0 + c;
        if (r >= nr || s >= ns)
            continue;
        const int f = (c + 2) * FR + RO + (q + 2);
        const unsigned int g = (unsigned int)s * pitch + (unsigned int)r;
        if constexpr (MODEL == 1) {
            const float ps = PSf[f];
            float fsum = 0.0f;
            for (int l = 0; l < L; ++l) {
                const float uc = div_cc<EXACT>(Uf[l * F + f], cc, inv_cc);
                const float dv = DV[l * R * S + i];
                const float ctv = CT[l * R * S + i];
                float p = (ps + uc) - dv;
                p = (p < ctv) ? p : ctv;
                d_pt[(unsigned int)l * lst + g] = p;
                const float ft = dv + p;
                DV[l * R * S + i] = ft;   // ft_l for the multipliers
                fsum += (ft - uc);
            }
            const float ps_n = (EXACT ? __fdiv_rn(fsum, (float)L) : fsum * (1.0f / (float)L)) +
                               P.inv_cc_l;
            d_ps[g] = ps_n;
            for (int l = 0; l < L; ++l) {
                const float e = cc * (DV[l * R * S + i] - ps_n);
                d_u[(unsigned int)l * lst + g] = Uf[l * F + f] - e;
                erru += abs_ref(e);
            }
        } else {
            float pt_below = 0.f, dv_below = 0.f, ucc_below = 0.f, u_below = 0.f;
            for (int l = 0; l < L; ++l) {
                float dv_l = 0.f, u_l = 0.f, ucc_l = 0.f, pt_up = 0.f;
                if (l < L - 1) {
                    dv_l = DV[l * R * S + i];
                    u_l = Uf[l * F + f];
                    ucc_l = div_cc<EXACT>(u_l, cc, inv_cc);
                    pt_up = PTf[(l + 1) * F + f];   // previous pt_{l+1}
                }
                float fpt;
                if (l == 0) {
                    fpt = ((dv_l + pt_up) - ucc_l) + inv_cc;
                } else if (l < L - 1) {
                    fpt = ((-dv_below) + pt_below) + ucc_below;
                    fpt = fpt + ((dv_l + pt_up) - ucc_l);
                    fpt = fpt * 0.5f;  // = fpt / 2 exactly
                } else {
                    fpt = ((-dv_below) + pt_below) + ucc_below;
                }
                const float pt_new = min_ref(fpt, CT[l * R * S + i]);
                d_pt[(unsigned int)l * lst + g] = pt_new;
                if (l >= 1) {
                    // multiplier of layer l-1 with the new pts
                    const float e = cc * ((dv_below + pt_new) - pt_below);
                    d_u[(unsigned int)(l - 1) * lst + g] = u_below - e;
                    erru += abs_ref(e);
                }
                pt_below = pt_new;
                dv_below = dv_l;
                ucc_below = ucc_l;
                u_below = u_l;
            }
        }
    }
    __syncthreads();  // the frame is reused by the next item or iteration
    return erru;
}

template <int MODEL, int NT, bool EXACT>
__global__ void __launch_bounds__(NT, 2) stencil2d_tile_labels_kernel(const __grid_constant__ BatchArgs B)
{
    extern __shared__ __align__(16) float fsm[];
    __shared__ double s_red[NT / 32];
    __shared__ int s_is_last;
    __shared__ int s_item;
    __shared__ int s_iter;
    const int tid = threadIdx.x;

    while (true) {
        if (tid == 0) {
            const int itm = (int)atomicAdd(&B.queue[0], 1u);
            int iter = -1;
            if (itm < B.total_items) {
                const IterControl *c = B.probs[B.item_problem[itm]].ctl;
                iter = *(const volatile int *)&c->done ? -1 : *(const volatile int *)&c->iter;
            }
            s_item = itm;
            s_iter = iter;
        }
        __syncthreads();
        const int item = s_item;
        const int it = s_iter;
        __syncthreads();  // s_item/s_iter are rewritten by the next fetch
        if (item >= B.total_items)
            break;
        if (it < 0)
            continue;  // the problem has converged
        const ProblemDesc &P = B.probs[B.item_problem[item]];
        const int li = item - P.item_begin;
        const float erru = ltile_iteration<MODEL, NT, EXACT>(P, it & 1, li, fsm);
        finish_item<NT>(erru, P, li, it, B.done_count, s_red, &s_is_last);
    }
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&B.queue[1], 1u) == gridDim.x - 1) {
            B.queue[0] = 0;
            B.queue[1] = 0;
            __threadfence();
        }
    }
}

// The whole solve in one cooperative launch, as stencil2d_tile_persistent_kernel.
template <int MODEL, int NT, bool EXACT>
__global__ void __launch_bounds__(NT, 2)
    stencil2d_tile_labels_persistent_kernel(const __grid_constant__ BatchArgs B)
{
    extern __shared__ __align__(16) float fsm[];
    __shared__ double s_red[NT / 32];
    __shared__ int s_stop;
    const ProblemDesc &P = B.probs[0];
    tile_solve_loop<NT>(P, B.queue, s_red, &s_stop, [&](int it, int tile) {
        return ltile_iteration<MODEL, NT, EXACT>(P, it & 1, tile, fsm);
    });
}

}  // namespace asets
