// One-pass iteration of the multi-label 2D solvers (Potts, Ishikawa): the
// flow update of every label and the per-pixel label update in one launch.
//
// The two-pass form (stencil2_kernel.cuh with the divergence epilogue, then
// label_kernels.cu) writes each label's divergence and re-reads it with pt
// and u.  Here a block owns a 60-row tile and a chunk of the stream axis
// (Matlab x) for ALL labels.  Flow warp k runs the column-per-thread step of
// stencil2_kernel.cuh for flow label k (two rows per thread, 64 rows per
// warp with two halo rows on each side, Lab2Flow below); where the two-pass
// form stores the divergence of plane s-2, the label update of that plane
// takes the values of all labels through shared memory:
//
//   Potts (maxflow/asetsPotts2D_mex.c:365-434): pt_k = min((ps + u_k/cc) -
//   dv_k, Ct_k), ft_k = dv_k + pt_k; ps = (sum over k, in label order, of
//   ft_k - u_k/cc) / L + 1/(cc L); u_k -= cc (ft_k - ps).
//   Ishikawa (maxflow/asetsIshikawa2D_mex.c:392-482): the ordered sink-flow
//   chain, lowest label first, then the multipliers.
//
// Two kernels share the flow step and differ in who runs the label update:
//
//   stencil2d_labels_kernel: one or two label warps, one step behind the
//   flow warps.  The flow warps hand plane s-2 over after the block barrier
//   of step t (Potts: after forming and storing pt_k); the label warps read
//   it after the barrier of step t+1, while the flow warps run the next
//   plane.  Double-buffered by step parity, one barrier per step.
//   stencil2d_labels_sync_kernel: the flow warps themselves, behind a second
//   barrier in the step (Potts: every warp sums the terms for its rows and
//   forms its own multiplier; Ishikawa: 64 threads run the chain).  Fewer
//   instructions, more waiting; the faster of the two depends on the size.
//
// Every array's labels come through one TMA box with a label extent (BR, BS,
// pt, u, alpha, Ct, and ps for Potts: 6-7 loads per plane); each flow thread
// keeps its own old u, pt (and ps) of the two planes behind in registers.
// The new pt, u and ps go to the other parity, as the flows do, because
// neighbouring blocks still read the old state as their halo.  Each value is
// the two-pass form's float expression in the same order, so EXACT results
// are bit-identical to it.
#pragma once

#include "stencil2_kernel.cuh"

namespace asets {

template <int MODEL, int L>
struct Lab2Geom {
    static_assert(MODEL == 1 || MODEL == 2, "Potts (1) or Ishikawa (2)");
    static constexpr int FL = (MODEL == 1) ? L : L - 1;   // flow labels = flow warps
    static_assert(FL >= 1 && FL <= 8, "one warp per flow label, at most 8");
    static constexpr int TR = 60;                         // tile rows
    static constexpr int LR = TR + 8;                     // halo box rows (origin r0-4)
    static constexpr int HAS_PS = (MODEL == 1) ? 1 : 0;
    static constexpr int slot_floats(int labels) { return (LR * labels + 31) & ~31; }  // 128 B
    // stage: BR[FL] | BS[FL] | PS[1] (Potts) | PT[L] | U[FL] | AL[FL] | CT[L] (three
    // planes behind: the plane whose labels step t updates or hands over)
    static constexpr int OFF_BR = 0;
    static constexpr int OFF_BS = OFF_BR + slot_floats(FL);
    static constexpr int OFF_PS = OFF_BS + slot_floats(FL);
    static constexpr int OFF_PT = OFF_PS + (HAS_PS ? slot_floats(1) : 0);
    static constexpr int OFF_U = OFF_PT + slot_floats(L);
    static constexpr int OFF_AL = OFF_U + slot_floats(FL);
    static constexpr int OFF_CT = OFF_AL + slot_floats(FL);
    static constexpr int STAGE = OFF_CT + slot_floats(L);         // floats
    static constexpr int TX = LR * 4 * (4 * FL + 2 * L + HAS_PS); // bytes per stage
    // label-warp hand-over buffer: [value][label][64 rows]; Potts term, ft,
    // u; Ishikawa dv, u, old pt_{k+1}, Ct and one more row for Ct_{L-1}
    static constexpr int XV = (MODEL == 1) ? 3 : 4;
    static constexpr int XBUF = (XV * FL + (MODEL == 1 ? 0 : 1)) * 64;  // floats
    // in-step exchange of the sync kernel: Potts the terms [FL][64];
    // Ishikawa dv [FL], u [FL], old pt [L] x 64 rows
    static constexpr int XSYNC = ((MODEL == 1) ? FL : 2 * FL + L) * 64;
};

// The TMA loads of one stage (its plane; Ct three planes behind).
template <int MODEL, int L>
__device__ __forceinline__ void lab2_issue(float *base, const ProblemDesc &P, int par, int r0,
                                           int plane, uint64_t *bar)
{
    using G = Lab2Geom<MODEL, L>;
    const CUtensorMap *hmaps = P.halo[par];
    mbar_arrive_expect_tx(bar, G::TX);
    tma_load_4d(base + G::OFF_BR, &hmaps[SL_BR], r0 - 4, 0, plane, 0, bar);
    tma_load_4d(base + G::OFF_BS, &hmaps[SL_BS], r0 - 4, 0, plane, 0, bar);
    if constexpr (MODEL == 1) {
        tma_load_4d(base + G::OFF_PS, &hmaps[SL_S0], r0 - 4, 0, plane, 0, bar);
        tma_load_4d(base + G::OFF_PT, &hmaps[SL_S1], r0 - 4, 0, plane, 0, bar);
    } else {
        tma_load_4d(base + G::OFF_PT, &hmaps[SL_S0], r0 - 4, 0, plane, 0, bar);
    }
    tma_load_4d(base + G::OFF_U, &hmaps[SL_S2], r0 - 4, 0, plane, 0, bar);
    tma_load_4d(base + G::OFF_AL, &hmaps[SL_ALPHA], r0 - 4, 0, plane, 0, bar);
    tma_load_4d(base + G::OFF_CT, &P.tile[par][TS_CT], r0 - 4, 0, plane - 3, 0, bar);
}

// A flow thread: rows r, r+1 of flow label k, swept along the stream axis.
// x_phase forms gk(s) from the stages of planes s and s+1; yz_phase the
// gradient step, the projection and the new faces of plane s-1 (stored) and
// returns the divergence of plane s-2; shift moves the thread's old u and
// ps (Potts) or pt_{k+1} (Ishikawa) down by one plane.
template <int MODEL, int L, bool EXACT>
struct Lab2Flow {
    using G = Lab2Geom<MODEL, L>;
    static constexpr int C = 2;
    static constexpr int LR = G::LR;
    int k, si;
    bool inplane[C], is_tile[C], fr_ok[C], fr1_ok[C];
    float fr_f[C], fr1_f[C];
    float gkprev[C], bsprev[C], g2prev[C], alpha_prev[C];
    float br_prev[C], bss_cur[C], bss_old[C], dvp[C];
    // old u_k, and ps (Potts) or pt_{k+1} (Ishikawa), of planes s-1 ([0]) and s-2 ([1])
    float f_u[2][C], f_a[2][C];
    // carried from x_phase to yz_phase and shift
    float gk[C], by_own[C], bs_own[C], alpha_cur[C], s0[C], s1[C], s2[C];

    __device__ __forceinline__ void init(int k_, int lane_row, int r, int nr)
    {
        k = k_;
        si = lane_row + 2;
        const bool tile_row = (lane_row >= 2 && lane_row < 62);
#pragma unroll
        for (int j = 0; j < C; ++j) {
            const int rj = r + j;
            inplane[j] = (rj >= 0 && rj < nr);
            is_tile[j] = tile_row && inplane[j];
            fr_ok[j] = (rj >= 1 && rj < nr);
            fr1_ok[j] = (rj + 1 >= 1 && rj + 1 < nr);
            fr_f[j] = fr_ok[j] ? 1.f : 0.f;
            fr1_f[j] = fr1_ok[j] ? 1.f : 0.f;
            gkprev[j] = bsprev[j] = br_prev[j] = bss_cur[j] = bss_old[j] = dvp[j] = 0.f;
            g2prev[j] = 1.f;
            alpha_prev[j] = 1.f;
            f_u[0][j] = f_u[1][j] = f_a[0][j] = f_a[1][j] = 0.f;
        }
    }

    __device__ __forceinline__ void x_phase(const float *stage_s, const float *stage_s1, float cc,
                                            float inv_cc)
    {
        const float *Sc = stage_s + si;
        const float *Sn = stage_s1 + si;
        float d[C], v[C];
        ld_cells<C>(Sc + G::OFF_BR + k * LR, by_own);
        d[0] = by_own[1] - by_own[0];
        d[1] = Sc[G::OFF_BR + k * LR + 2] - by_own[1];
        ld_cells<C>(Sc + G::OFF_BS + k * LR, bs_own);
        ld_cells<C>(Sn + G::OFF_BS + k * LR, v);
#pragma unroll
        for (int j = 0; j < C; ++j) {
            d[j] = d[j] + v[j];
            d[j] = d[j] - bs_own[j];
        }
        if constexpr (MODEL == 1) {
            ld_cells<C>(Sc + G::OFF_PS, s0);                  // ps
            ld_cells<C>(Sc + G::OFF_PT + k * LR, s1);         // pt_k
        } else {
            ld_cells<C>(Sc + G::OFF_PT + k * LR, s0);         // pt_k
            ld_cells<C>(Sc + G::OFF_PT + (k + 1) * LR, s1);   // pt_{k+1}
        }
        ld_cells<C>(Sc + G::OFF_U + k * LR, s2);              // u_k
#pragma unroll
        for (int j = 0; j < C; ++j)
            gk[j] = d[j] - ((s0[j] - s1[j]) + div_cc<EXACT>(s2[j], cc, inv_cc));
        ld_cells<C>(Sc + G::OFF_AL + k * LR, alpha_cur);
    }

    // b'(s), g2(s-1), b''(s-1) (stored when plane s-1 is the item's); dv(s-2)
    __device__ __forceinline__ void yz_phase(int s, int ns, int s_begin, int s_end, float steps,
                                             float *__restrict__ d_bs, float *__restrict__ d_br,
                                             unsigned int off_sp, const ProblemDesc &P, float (&dv)[C])
    {
        const bool s_in = (s >= 0 && s < ns);
        const bool sb_in = (s >= 1 && s < ns);          // stream face s is interior
        const bool sp_in = (s - 1 >= 0 && s - 1 < ns);
        const bool spb_in = (s - 1 >= 1 && s - 1 < ns);
        const float sb_f = sb_in ? 1.f : 0.f, spb_f = spb_in ? 1.f : 0.f;
        const bool sp_out = (s - 1 >= s_begin && s - 1 < s_end);
        float gk_up[C], brn[C], bsn[C], br_dn[C], g2[C], bssn[C];
        rows_up<C>(gk, gk_up);
#pragma unroll
        for (int j = 0; j < C; ++j) {
            brn[j] = keep_if<EXACT>(steps * (gk[j] - gk_up[j]) + by_own[j], fr_ok[j] && s_in,
                                    fr_f[j]);
            bsn[j] = keep_if<EXACT>(steps * (gk[j] - gkprev[j]) + bs_own[j], inplane[j] && sb_in,
                                    sb_f);
            gkprev[j] = gk[j];
        }
        rows_down<C>(br_prev, br_dn);   // b'_r(s-1) at r+1
#pragma unroll
        for (int j = 0; j < C; ++j)
            g2[j] = Proj<EXACT>::gk(bsn[j], bsprev[j], br_dn[j], br_prev[j], alpha_prev[j]);
#pragma unroll
        for (int j = 0; j < C; ++j) {
            bssn[j] = keep_if<EXACT>(((g2[j] + g2prev[j]) * 0.5f) * bsprev[j], inplane[j] && spb_in,
                                     spb_f);
            bss_old[j] = bss_cur[j];
            bss_cur[j] = bssn[j];
            g2prev[j] = g2[j];
            bsprev[j] = bsn[j];
            alpha_prev[j] = alpha_cur[j];
        }
        if (sp_out)
            st_dst<C>(d_bs, off_sp, bssn, is_tile, P);
        // row faces b''_r(s-1), the divergence of plane s-2
        float g2_up[C], g2_dn[C], brr[C], dn[C];
        rows_up<C>(g2, g2_up);
        rows_down<C>(g2, g2_dn);
#pragma unroll
        for (int j = 0; j < C; ++j) {
            brr[j] = keep_if<EXACT>(((g2[j] + g2_up[j]) * 0.5f) * br_prev[j], fr_ok[j] && sp_in,
                                    fr_f[j]);
            const float brr1 = keep_if<EXACT>(((g2_dn[j] + g2[j]) * 0.5f) * br_dn[j],
                                              fr1_ok[j] && sp_in, fr1_f[j]);
            dn[j] = brr1 - brr[j];
        }
        if (sp_out)
            st_dst<C>(d_br, off_sp, brr, is_tile, P);
#pragma unroll
        for (int j = 0; j < C; ++j) {
            dv[j] = dvp[j] + bss_cur[j];
            dv[j] = dv[j] - bss_old[j];
            dvp[j] = dn[j];
            br_prev[j] = brn[j];
        }
    }

    __device__ __forceinline__ void shift()
    {
#pragma unroll
        for (int j = 0; j < C; ++j) {
            f_u[1][j] = f_u[0][j];
            f_u[0][j] = s2[j];
            f_a[1][j] = f_a[0][j];
            f_a[0][j] = (MODEL == 1) ? s0[j] : s1[j];   // ps, or pt_{k+1}
        }
    }
};

// Potts: pt_k of plane s-2 from the thread's old ps and u_k and its Ct; the
// term ft_k - u_k/cc of the source-flow sum and ft_k.
template <bool EXACT>
__device__ __forceinline__ void potts_pt(const float (&ps)[2], const float (&u)[2],
                                         const float (&dv)[2], const float (&ct)[2], float cc,
                                         float inv_cc, float (&pt)[2], float (&ft)[2],
                                         float (&term)[2])
{
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const float uc = div_cc<EXACT>(u[j], cc, inv_cc);
        const float p = (ps[j] + uc) - dv[j];
        pt[j] = (p < ct[j]) ? p : ct[j];
        ft[j] = dv[j] + pt[j];
        term[j] = ft[j] - uc;
    }
}

// Ishikawa: layer l of the ordered chain for one pixel (the layer below in
// pt_below, dv_below, ucc_below).  Returns the new pt_l and, in *e, the
// multiplier change of layer l-1 (meaningful for l >= 1).
template <bool EXACT, int L>
__device__ __forceinline__ float ishikawa_layer(int l, float dv_l, float ucc_l, float pt_up,
                                                float ctv, float pt_below, float dv_below,
                                                float ucc_below, float cc, float inv_cc, float *e)
{
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
    const float pt_new = min_ref(fpt, ctv);
    // multiplier of layer l-1 with the new pts
    *e = cc * ((dv_below + pt_new) - pt_below);
    return pt_new;
}

// Claim the next item of the launch: thread 0 reads its problem's iteration
// once for the block.  Returns false when the launch has no items left.
__device__ __forceinline__ bool lab2_next_item(const BatchArgs &B, int *s_item, int *s_iter,
                                               int &item, int &it)
{
    if (threadIdx.x == 0) {
        const int itm = (int)atomicAdd(&B.queue[0], 1u);
        int iter = -1;
        if (itm < B.total_items) {
            const IterControl *c = B.probs[B.item_problem[itm]].ctl;
            iter = *(const volatile int *)&c->done ? -1 : *(const volatile int *)&c->iter;
        }
        *s_item = itm;
        *s_iter = iter;
    }
    __syncthreads();
    item = *s_item;
    it = *s_iter;
    __syncthreads();  // s_item/s_iter are rewritten by the next fetch
    return item < B.total_items;
}

// the last block to leave re-arms the queue for the next launch
__device__ __forceinline__ void lab2_leave(const BatchArgs &B)
{
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&B.queue[1], 1u) == gridDim.x - 1) {
            B.queue[0] = 0;
            B.queue[1] = 0;
            __threadfence();
        }
    }
}

// ---------------------------------------------------------------- label warps
template <int MODEL, int L, int LW>
struct Lab2WarpsGeom {
    using G = Lab2Geom<MODEL, L>;
    static_assert(LW == 1 || LW == 2, "one label warp (two rows a thread) or two (one row)");
    static constexpr int NW = G::FL + LW;
    static constexpr int NT = 32 * NW;
    static constexpr int LC = 2 / LW;   // rows a label-warp thread updates
    template <int NSTAGE>
    static constexpr int smem_bytes() { return (NSTAGE * G::STAGE + 2 * G::XBUF) * 4 + NSTAGE * 8 + 128; }
};

template <int MODEL, int L, int LW, int NSTAGE, bool EXACT, int MINB>
__global__ void __launch_bounds__(32 * Lab2WarpsGeom<MODEL, L, LW>::NW, MINB)
    stencil2d_labels_kernel(const __grid_constant__ BatchArgs B)
{
    using G = Lab2Geom<MODEL, L>;
    using W = Lab2WarpsGeom<MODEL, L, LW>;
    constexpr int FL = G::FL;
    constexpr int NT = W::NT;
    constexpr int LC = W::LC;
    constexpr int C = 2;
    static_assert(NSTAGE >= 4, "stage of plane s stays resident until step s ends");

    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ int s_abort;
    __shared__ double s_red[NT / 32];
    __shared__ int s_is_last;
    __shared__ int s_item;
    __shared__ int s_iter;

    const int tid = threadIdx.x, lane = tid & 31, k = tid >> 5;  // flow warp k = flow label k
    const bool flow = (k < FL);                                  // warps FL..: the label warps
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
    float *stages = reinterpret_cast<float *>(smem);
    float *xch = stages + NSTAGE * G::STAGE;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + (NSTAGE * G::STAGE + 2 * G::XBUF) * 4);

    for (int i = tid; i < 2 * G::XBUF; i += NT)
        xch[i] = 0.f;
    if (tid == 0) {
        s_abort = 0;
        for (int i = 0; i < NSTAGE; ++i)
            mbar_init(&bars[i], 1);
        mbar_fence_init();
    }
    __syncthreads();

    const int lane_row = C * lane;                  // a flow thread's rows within the 64
    const bool producer = (tid == FL * 32);         // lane 0 of the first label warp
    // a label-warp thread's rows within the 64: two (one label warp) or one
    const int lab_row = (LW == 1) ? lane_row : (k - FL) * 32 + lane;
    // hand-over entry (value v, label l) of buffer b at row `row`
    auto xat = [&](int b, int v, int l, int row) { return xch + b * G::XBUF + (v * FL + l) * 64 + row; };

    unsigned int q0 = 0;
    bool aborted = false;
    int item, it;
    while (!aborted && lab2_next_item(B, &s_item, &s_iter, item, it)) {
        if (it < 0)
            continue;  // the problem has converged
        const ProblemDesc &P = B.probs[B.item_problem[item]];
        const int par = it & 1;
        const int nr = P.nr, ns = P.ns;
        const float cc = P.cc, inv_cc = P.inv_cc, steps = P.steps;
        const int li = item - P.item_begin;
        // chunk-major order: neighbouring tiles of one chunk run together
        const int tile = li % P.tiles_r;
        const int chunk = li / P.tiles_r;
        const int s_begin = (int)((long long)ns * chunk / P.zchunks);
        const int s_end = (int)((long long)ns * (chunk + 1) / P.zchunks);
        const int r0 = tile * G::TR;
        const int n_steps = s_end - s_begin + 4;
        const int n_loads = n_steps + 1;
        const int p_first = s_begin - 2;
        float erru = 0.0f;

        auto issue_load = [&](int j) {
            const unsigned int q = q0 + j;
            lab2_issue<MODEL, L>(stages + (q % NSTAGE) * G::STAGE, P, par, r0, p_first + j,
                                 &bars[q % NSTAGE]);
        };
        if (producer)
            for (int j = 0; j < NSTAGE && j < n_loads; ++j)
                issue_load(j);

        // element offsets fit 32 bits: solves are limited to 2^32 padded voxel-labels
        const unsigned int S = (unsigned int)P.label_stride;
        const unsigned int plane_stride = (unsigned int)P.plane_stride;
        const int r = r0 - 2 + lane_row;
        const unsigned int col_off = (unsigned int)k * S + (unsigned int)r;  // flow warps
        float *__restrict__ d_bs = P.dst_b[par][SL_BS];
        float *__restrict__ d_br = P.dst_b[par][SL_BR];
        // the new state goes to the other parity: Potts ps, pt, u; Ishikawa pt, -, u
        float *__restrict__ d_s0 = P.dst_s[par][0];
        float *__restrict__ d_s1 = P.dst_s[par][1];
        float *__restrict__ d_s2 = P.dst_s[par][2];
        Lab2Flow<MODEL, L, EXACT> F;
        F.init(k, lane_row, r, nr);
        // halo-box reads si .. si+C of a label's LR rows
        check_index(F.si + C, G::LR, P);

        // the label-warp thread's rows r0-2+lab_row .. +LC-1: in the tile?
        bool lab_ok[LC];
#pragma unroll
        for (int j = 0; j < LC; ++j)
            lab_ok[j] = (lab_row + j >= 2 && lab_row + j < 62 && r0 - 2 + lab_row + j < nr);

        // The label warps' update of plane pl from hand-over buffer b.
        auto label_update = [&](int b, int pl) {
            const bool pl_out = (pl >= s_begin && pl < s_end);
            const unsigned int o = (unsigned int)(r0 - 2 + lab_row) + (unsigned int)pl * plane_stride;
            if constexpr (MODEL == 1) {
                float fsum[LC], ps_n[LC];
#pragma unroll
                for (int j = 0; j < LC; ++j)
                    fsum[j] = 0.0f;
#pragma unroll
                for (int l = 0; l < L; ++l) {
                    float term[LC];
                    ld_cells<LC>(xat(b, 0, l, lab_row), term);
#pragma unroll
                    for (int j = 0; j < LC; ++j)
                        fsum[j] += term[j];
                }
#pragma unroll
                for (int j = 0; j < LC; ++j)
                    ps_n[j] = (EXACT ? __fdiv_rn(fsum[j], (float)L) : fsum[j] * (1.0f / (float)L)) +
                              P.inv_cc_l;
                if (pl_out)
                    st_dst<LC>(d_s0, o, ps_n, lab_ok, P);
#pragma unroll
                for (int l = 0; l < L; ++l) {
                    float ft[LC], u[LC], un[LC];
                    ld_cells<LC>(xat(b, 1, l, lab_row), ft);
                    ld_cells<LC>(xat(b, 2, l, lab_row), u);
#pragma unroll
                    for (int j = 0; j < LC; ++j) {
                        const float e = cc * (ft[j] - ps_n[j]);
                        un[j] = u[j] - e;
                        if (pl_out && lab_ok[j])
                            erru += abs_ref(e);
                    }
                    if (pl_out)
                        st_dst<LC>(d_s2, o + (unsigned int)l * S, un, lab_ok, P);
                }
            } else {
                // the sink-flow chain, lowest label first, LC pixels at a time
                float pt_below[LC], dv_below[LC], ucc_below[LC], u_below[LC];
#pragma unroll
                for (int j = 0; j < LC; ++j)
                    pt_below[j] = dv_below[j] = ucc_below[j] = u_below[j] = 0.f;
#pragma unroll
                for (int l = 0; l < L; ++l) {
                    float dv_l[LC], u_l[LC], ucc_l[LC], pt_up[LC], ctv[LC], pt_new[LC], un[LC];
#pragma unroll
                    for (int j = 0; j < LC; ++j)
                        dv_l[j] = u_l[j] = ucc_l[j] = pt_up[j] = 0.f;
                    if (l < L - 1) {
                        ld_cells<LC>(xat(b, 0, l, lab_row), dv_l);
                        ld_cells<LC>(xat(b, 1, l, lab_row), u_l);
                        ld_cells<LC>(xat(b, 2, l, lab_row), pt_up);   // previous pt_{l+1}
                        ld_cells<LC>(xat(b, 3, l, lab_row), ctv);
                    } else {
                        ld_cells<LC>(xat(b, 4, 0, lab_row), ctv);     // Ct_{L-1}
                    }
#pragma unroll
                    for (int j = 0; j < LC; ++j) {
                        if (l < L - 1)
                            ucc_l[j] = div_cc<EXACT>(u_l[j], cc, inv_cc);
                        float e;
                        pt_new[j] = ishikawa_layer<EXACT, L>(l, dv_l[j], ucc_l[j], pt_up[j], ctv[j],
                                                             pt_below[j], dv_below[j], ucc_below[j],
                                                             cc, inv_cc, &e);
                        un[j] = u_below[j] - e;
                        if (l >= 1 && pl_out && lab_ok[j])
                            erru += abs_ref(e);
                    }
                    if (pl_out) {
                        st_dst<LC>(d_s0, o + (unsigned int)l * S, pt_new, lab_ok, P);
                        if (l >= 1)
                            st_dst<LC>(d_s2, o + (unsigned int)(l - 1) * S, un, lab_ok, P);
                    }
#pragma unroll
                    for (int j = 0; j < LC; ++j) {
                        pt_below[j] = pt_new[j];
                        dv_below[j] = dv_l[j];
                        ucc_below[j] = ucc_l[j];
                        u_below[j] = u_l[j];
                    }
                }
            }
        };

        // A wait gave up: drain this item's loads [first, issued) (bounded),
        // record the error and leave the item.
        auto abort_item = [&](int first, int issued) {
            if (producer) {
                s_abort = 0;
                for (int j = first; j < issued; ++j) {
                    const unsigned int q = q0 + j;
                    mbar_wait_bounded(&bars[q % NSTAGE], (q / NSTAGE) & 1, &s_abort);
                }
                atomicOr(&P.ctl->error, DEV_ERR_TIMEOUT);
            }
            __syncthreads();
        };

        // Step t: the flow warps read the stages of planes t and t+1 (X, and
        // Ct after the barrier) and fill hand-over buffer t&1; the label
        // warps read buffer (t-1)&1, filled before this step's barrier.
        // After the barrier stage t is refilled with plane t+NSTAGE.
        for (int t = 0; t < n_steps && !aborted; ++t) {
            const int s = p_first + t;
            const int st_cur = (q0 + t) % NSTAGE, st_nxt = (q0 + t + 1) % NSTAGE;
            bool wait_ok = true;
            if (flow) {
                if (t == 0)
                    wait_ok = mbar_wait_bounded(&bars[st_cur], ((q0 + t) / NSTAGE) & 1, &s_abort);
                wait_ok = wait_ok && mbar_wait_bounded(&bars[st_nxt], ((q0 + t + 1) / NSTAGE) & 1,
                                                        &s_abort);
                F.x_phase(stages + st_cur * G::STAGE, stages + st_nxt * G::STAGE, cc, inv_cc);
            }
            if (__syncthreads_or(!wait_ok)) {
                aborted = true;
                // loads issued: the prologue, then one per earlier step
                abort_item(t, min(n_loads, t + NSTAGE));
                break;
            }
            if (producer && t + NSTAGE < n_loads)
                issue_load(t + NSTAGE);
            if (!flow) {
                label_update((t - 1) & 1, s - 3);   // handed over last step
                continue;
            }
            float dv[C];
            F.yz_phase(s, ns, s_begin, s_end, steps, d_bs, d_br,
                       col_off + (unsigned int)(s - 1) * plane_stride, P, dv);

            // ---- hand plane so = s-2 over (its Ct came with the stage of plane s+1)
            const int so = s - 2;
            const float *CT = stages + st_nxt * G::STAGE + G::OFF_CT + F.si;
            const int b = t & 1;
            float ct[C];
            ld_cells<C>(CT + k * G::LR, ct);
            if constexpr (MODEL == 1) {
                float pt[C], ft[C], term[C];
                potts_pt<EXACT>(F.f_a[1], F.f_u[1], dv, ct, cc, inv_cc, pt, ft, term);
                if (so >= s_begin && so < s_end)
                    st_dst<C>(d_s1, col_off + (unsigned int)so * plane_stride, pt, F.is_tile, P);
                st_cells<C>(xat(b, 0, k, lane_row), term);
                st_cells<C>(xat(b, 1, k, lane_row), ft);
                st_cells<C>(xat(b, 2, k, lane_row), F.f_u[1]);
            } else {
                st_cells<C>(xat(b, 0, k, lane_row), dv);
                st_cells<C>(xat(b, 1, k, lane_row), F.f_u[1]);
                st_cells<C>(xat(b, 2, k, lane_row), F.f_a[1]);   // old pt_{k+1}
                st_cells<C>(xat(b, 3, k, lane_row), ct);
                if (k == FL - 1) {
                    float ctl[C];
                    ld_cells<C>(CT + (L - 1) * G::LR, ctl);
                    st_cells<C>(xat(b, 4, 0, lane_row), ctl);
                }
            }
            F.shift();
        }
        q0 += n_loads;
        __syncthreads();  // the last step's hand-over is written; stages are free
        if (!aborted && !flow)
            label_update((n_steps - 1) & 1, p_first + n_steps - 3);
        finish_item<NT>(erru, P, li, it, B.done_count, s_red, &s_is_last);
    }
    lab2_leave(B);
}

// ---------------------------------------------------------------- in-step update
template <int MODEL, int L>
struct Lab2SyncGeom {
    using G = Lab2Geom<MODEL, L>;
    static constexpr int NW = G::FL;
    static constexpr int NT = 32 * NW;
    template <int NSTAGE>
    static constexpr int smem_bytes() { return (NSTAGE * G::STAGE + G::XSYNC) * 4 + NSTAGE * 8 + 128; }
};

template <int MODEL, int L, int NSTAGE, bool EXACT, int MINB>
__global__ void __launch_bounds__(32 * Lab2Geom<MODEL, L>::FL, MINB)
    stencil2d_labels_sync_kernel(const __grid_constant__ BatchArgs B)
{
    using G = Lab2Geom<MODEL, L>;
    constexpr int FL = G::FL;
    constexpr int NT = Lab2SyncGeom<MODEL, L>::NT;
    constexpr int C = 2;
    static_assert(NSTAGE >= 4, "stage of plane s stays resident until step s ends");

    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ int s_abort;
    __shared__ double s_red[NT / 32];
    __shared__ int s_is_last;
    __shared__ int s_item;
    __shared__ int s_iter;

    const int tid = threadIdx.x, lane = tid & 31, k = tid >> 5;  // warp = flow label
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
    float *stages = reinterpret_cast<float *>(smem);
    float *X = stages + NSTAGE * G::STAGE;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + (NSTAGE * G::STAGE + G::XSYNC) * 4);

    if (tid == 0) {
        s_abort = 0;
        for (int i = 0; i < NSTAGE; ++i)
            mbar_init(&bars[i], 1);
        mbar_fence_init();
    }
    __syncthreads();

    const int lane_row = C * lane;                  // the thread's rows within the 64
    const bool producer = (tid == NT - 32);

    unsigned int q0 = 0;
    bool aborted = false;
    int item, it;
    while (!aborted && lab2_next_item(B, &s_item, &s_iter, item, it)) {
        if (it < 0)
            continue;  // the problem has converged
        const ProblemDesc &P = B.probs[B.item_problem[item]];
        const int par = it & 1;
        const int nr = P.nr, ns = P.ns;
        const float cc = P.cc, inv_cc = P.inv_cc, steps = P.steps;
        const int li = item - P.item_begin;
        const int tile = li % P.tiles_r;
        const int chunk = li / P.tiles_r;
        const int s_begin = (int)((long long)ns * chunk / P.zchunks);
        const int s_end = (int)((long long)ns * (chunk + 1) / P.zchunks);
        const int r0 = tile * G::TR;
        const int n_steps = s_end - s_begin + 4;
        const int n_loads = n_steps + 1;
        const int p_first = s_begin - 2;
        float erru = 0.0f;

        auto issue_load = [&](int j) {
            const unsigned int q = q0 + j;
            lab2_issue<MODEL, L>(stages + (q % NSTAGE) * G::STAGE, P, par, r0, p_first + j,
                                 &bars[q % NSTAGE]);
        };
        if (producer)
            for (int j = 0; j < NSTAGE && j < n_loads; ++j)
                issue_load(j);

        const unsigned int S = (unsigned int)P.label_stride;
        const unsigned int plane_stride = (unsigned int)P.plane_stride;
        const int r = r0 - 2 + lane_row;
        const unsigned int col_off = (unsigned int)k * S + (unsigned int)r;
        float *__restrict__ d_bs = P.dst_b[par][SL_BS];
        float *__restrict__ d_br = P.dst_b[par][SL_BR];
        float *__restrict__ d_s0 = P.dst_s[par][0];
        float *__restrict__ d_s1 = P.dst_s[par][1];
        float *__restrict__ d_s2 = P.dst_s[par][2];
        Lab2Flow<MODEL, L, EXACT> F;
        F.init(k, lane_row, r, nr);
        check_index(F.si + C, G::LR, P);

        auto abort_item = [&](int first, int issued) {
            if (producer) {
                s_abort = 0;
                for (int j = first; j < issued; ++j) {
                    const unsigned int q = q0 + j;
                    mbar_wait_bounded(&bars[q % NSTAGE], (q / NSTAGE) & 1, &s_abort);
                }
                atomicOr(&P.ctl->error, DEV_ERR_TIMEOUT);
            }
            __syncthreads();
        };

        // Step t reads the stages of planes t and t+1; after the X barrier
        // stage t is refilled with plane t+NSTAGE.  The exchange is written
        // after the X barrier and read after the exchange barrier of the
        // same step, so one buffer serves every step.
        for (int t = 0; t < n_steps && !aborted; ++t) {
            const int s = p_first + t;
            const int st_cur = (q0 + t) % NSTAGE, st_nxt = (q0 + t + 1) % NSTAGE;
            bool wait_ok = true;
            if (t == 0)
                wait_ok = mbar_wait_bounded(&bars[st_cur], ((q0 + t) / NSTAGE) & 1, &s_abort);
            wait_ok = wait_ok && mbar_wait_bounded(&bars[st_nxt], ((q0 + t + 1) / NSTAGE) & 1,
                                                    &s_abort);
            F.x_phase(stages + st_cur * G::STAGE, stages + st_nxt * G::STAGE, cc, inv_cc);
            if (__syncthreads_or(!wait_ok)) {
                aborted = true;
                abort_item(t, min(n_loads, t + NSTAGE));
                break;
            }
            if (producer && t + NSTAGE < n_loads)
                issue_load(t + NSTAGE);
            float dv[C];
            F.yz_phase(s, ns, s_begin, s_end, steps, d_bs, d_br,
                       col_off + (unsigned int)(s - 1) * plane_stride, P, dv);

            // ---- the label update of plane so = s-2 (Ct from the stage of plane s+1)
            const int so = s - 2;
            const bool so_out = (so >= s_begin && so < s_end);
            const unsigned int o = col_off + (unsigned int)so * plane_stride;
            const float *CT = stages + st_nxt * G::STAGE + G::OFF_CT;
            if constexpr (MODEL == 1) {
                float ct[C], pt[C], ft[C], term[C];
                ld_cells<C>(CT + k * G::LR + F.si, ct);
                potts_pt<EXACT>(F.f_a[1], F.f_u[1], dv, ct, cc, inv_cc, pt, ft, term);
                st_cells<C>(X + k * 64 + lane_row, term);
                __syncthreads();
                float ps_n[C], u_n[C];
#pragma unroll
                for (int j = 0; j < C; ++j) {
                    float fsum = 0.0f;
#pragma unroll
                    for (int l = 0; l < L; ++l)
                        fsum += X[l * 64 + lane_row + j];
                    ps_n[j] = (EXACT ? __fdiv_rn(fsum, (float)L) : fsum * (1.0f / (float)L)) +
                              P.inv_cc_l;
                    const float e = cc * (ft[j] - ps_n[j]);
                    u_n[j] = F.f_u[1][j] - e;
                    if (so_out && F.is_tile[j])
                        erru += abs_ref(e);
                }
                if (so_out) {
                    st_dst<C>(d_s1, o, pt, F.is_tile, P);
                    st_dst<C>(d_s2, o, u_n, F.is_tile, P);
                    if (k == 0)
                        st_dst<C>(d_s0, o, ps_n, F.is_tile, P);  // ps: label 0's offsets
                }
            } else {
                // share dv_k, u_k and the old pt_{k+1}
                st_cells<C>(X + k * 64 + lane_row, dv);
                st_cells<C>(X + (FL + k) * 64 + lane_row, F.f_u[1]);
                st_cells<C>(X + (2 * FL + k + 1) * 64 + lane_row, F.f_a[1]);
                __syncthreads();
                // one pixel per thread (row r0-2+q), labels lowest first; a
                // one-warp block takes two
                for (int q = tid; q < 64; q += NT) {
                    const int rr = r0 - 2 + q;
                    const bool mine = so_out && q >= 2 && q < 62 && rr < nr;
                    const unsigned int og = (unsigned int)rr + (unsigned int)so * plane_stride;
                    float pt_below = 0.f, dv_below = 0.f, ucc_below = 0.f, u_below = 0.f;
#pragma unroll
                    for (int l = 0; l < L; ++l) {
                        float dv_l = 0.f, u_l = 0.f, ucc_l = 0.f, pt_up = 0.f;
                        if (l < L - 1) {
                            dv_l = X[l * 64 + q];
                            u_l = X[(FL + l) * 64 + q];
                            ucc_l = div_cc<EXACT>(u_l, cc, inv_cc);
                            pt_up = X[(2 * FL + l + 1) * 64 + q];  // previous pt_{l+1}
                        }
                        float e;
                        const float pt_new = ishikawa_layer<EXACT, L>(
                            l, dv_l, ucc_l, pt_up, CT[l * G::LR + q + 2], pt_below, dv_below,
                            ucc_below, cc, inv_cc, &e);
                        if (mine) {
                            d_s0[og + (unsigned int)l * S] = pt_new;
                            if (l >= 1) {
                                d_s2[og + (unsigned int)(l - 1) * S] = u_below - e;
                                erru += abs_ref(e);
                            }
                        }
                        pt_below = pt_new;
                        dv_below = dv_l;
                        ucc_below = ucc_l;
                        u_below = u_l;
                    }
                }
            }
            F.shift();
        }
        q0 += n_loads;
        __syncthreads();  // stage slots and the exchange buffer are reused by the next item
        finish_item<NT>(erru, P, li, it, B.done_count, s_red, &s_is_last);
    }
    lab2_leave(B);
}

}  // namespace asets
