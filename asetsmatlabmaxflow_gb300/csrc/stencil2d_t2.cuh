// Two ALM iterations per pass of the binary 2D solver (temporal blocking).
//
// One launch performs iterations it and it+1 of every problem in it.  The
// first iteration (A) is the column-per-thread step of stencil2_kernel.cuh
// on the old state staged by TMA; the second (B) runs the same step two
// planes behind A on A's results, which never leave the registers: A's new
// row faces r and r+1 (from A's previous step), its stream faces of the
// current and the previous step and its ps/pt/u (just computed).  Only B's
// state is written, so a pass moves the bytes of one iteration for two.
//
// Geometry.  Each warp owns 64 consecutive rows (two per thread): A's
// results are valid on rows 2..61 of them, B's on rows 4..59, so a warp's
// output tile is 56 rows and the NW warps stack to TR = 56*NW tile rows.
// The halo box spans rows r0-4 .. r0+TR+8 (the warps' rows plus the row
// face below the last one), the tile boxes (old pt and u, Cs, Ct of the
// plane A's epilogue writes) rows r0-4 .. r0+TR+4.  Along the stream axis
// (x in 2D) a chunk of output planes [s_begin, s_end) needs A on
// [s_begin-2, s_end+2) and so reads [s_begin-4, s_end+4): 8 warm-up steps.
//
// State outside the image is zero in the single-iteration kernel (the tile
// loads' out-of-range fill); here A's ps/pt/u outside the image are set to
// zero before B reads them, and A's flows there come out zero by the same
// masks as in stencil2_kernel.cuh.  Every value B computes is the same
// float expression, in the same order, as the single-iteration kernel's,
// so EXACT results are bit-identical to two single iterations.
//
// erriter: each item sums |e| of both iterations over its output cells;
// the last item of the problem's pair writes cvg[it] and cvg[it+1].  When
// iteration it already meets errBound (or is the last of maxIt) the pass
// has gone one iteration too far: the control block records `rollback` and
// the host re-runs that iteration alone from the state before the pass.
#pragma once

#include "stencil2_kernel.cuh"

namespace asets {

template <int NW>
struct T2Geom {
    static constexpr int NT = 32 * NW;
    static constexpr int TRW = 56;                 // output rows per warp
    static constexpr int TR = TRW * NW;            // tile rows
    static constexpr int LR = TR + 12;             // halo box rows (origin r0-4)
    static constexpr int TB = TR + 8;              // tile box rows (origin r0-4)
    static_assert(LR <= 256, "TMA box dimension limit");
    static constexpr int align128(int b) { return (b + 127) & ~127; }
    static constexpr int halo_slot_bytes() { return align128(LR * 4); }
    static constexpr int tile_slot_bytes() { return align128(TB * 4); }
    // six halo slots (no column faces in 2D) and four tile slots
    static constexpr int stage_bytes() { return 6 * halo_slot_bytes() + 4 * tile_slot_bytes(); }
    static constexpr int tx_bytes() { return 6 * LR * 4 + 4 * TB * 4; }
    template <int NSTAGE>
    static constexpr int smem_bytes() { return NSTAGE * stage_bytes() + NSTAGE * 8 + 128; }
};

// Both iterations' erriter partials of an item, then the last item of the
// problem's pass closes iterations it and it+1 (see the header).
template <int NT>
__device__ __forceinline__ void finish_item_t2(float erru_a, float erru_b, const ProblemDesc &P,
                                               int li, int it, unsigned int *done_count,
                                               double *s_red, int *s_is_last)
{
    const double pa = block_sum_double<NT>(erru_a, s_red);
    __syncthreads();
    const double pb = block_sum_double<NT>(erru_b, s_red);
    IterControl *ctl = P.ctl;
    if (threadIdx.x == 0) {
        P.item_partials[2 * li] = pa;
        P.item_partials[2 * li + 1] = pb;
        __threadfence();
        const unsigned int ticket = atomicAdd(&ctl->ticket, 1u);
        *s_is_last = (ticket == (unsigned int)P.n_items - 1);
    }
    __syncthreads();
    if (*s_is_last && threadIdx.x < 32) {
        __threadfence();
        double acc_a = 0.0, acc_b = 0.0;
        for (int b = threadIdx.x; b < P.n_items; b += 32) {
            acc_a += __ldcg(P.item_partials + 2 * b);
            acc_b += __ldcg(P.item_partials + 2 * b + 1);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            acc_a += __shfl_xor_sync(0xffffffffu, acc_a, o);
            acc_b += __shfl_xor_sync(0xffffffffu, acc_b, o);
        }
        if (threadIdx.x == 0) {
            auto meets = [&](float c) {
                return ctl->break_lt ? (c < ctl->err_bound) : (c <= ctl->err_bound);
            };
            int done = 0;
            const float ca = __fdiv_rn((float)acc_a, ctl->denom);
            P.cvg[it] = ca;
            if (ctl->error || meets(ca) || it + 1 >= ctl->max_it) {
                // iteration it ends the solve: its state is the result
                done = 1;
                ctl->it_num = (ctl->error || meets(ca)) ? it : ctl->max_it;
                ctl->last_iter = it;
                ctl->rollback = 1;
            } else {
                const float cb = __fdiv_rn((float)acc_b, ctl->denom);
                P.cvg[it + 1] = cb;
                ctl->last_iter = it + 1;
                if (meets(cb)) {
                    done = 1;
                    ctl->it_num = it + 1;
                } else if (it + 2 >= ctl->max_it) {
                    done = 1;
                    ctl->it_num = ctl->max_it;
                }
            }
            ctl->ticket = 0;
            ctl->iter = it + 2;
            if (done) {
                ctl->done = 1;
                atomicAdd(done_count, 1u);
            }
            __threadfence();
        }
    }
    __syncthreads();
}

template <int NW, int NSTAGE, bool EXACT, int MINB, int UNROLL = 1>
__global__ void __launch_bounds__(32 * NW, MINB)
    stencil2d_t2_kernel(const __grid_constant__ BatchArgs B)
{
    using G = T2Geom<NW>;
    constexpr int NT = G::NT;
    constexpr int C = 2;
    static_assert(NSTAGE >= 4, "stage of plane s stays resident until step s ends");

    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ int s_abort;
    __shared__ double s_red[NT / 32];
    __shared__ int s_is_last;
    __shared__ int s_item;
    __shared__ int s_iter;

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
    constexpr int SB = G::stage_bytes();
    constexpr int HS = G::halo_slot_bytes() / 4;   // floats per halo slot
    constexpr int TS = G::tile_slot_bytes() / 4;   // floats per tile slot
    // halo slot order in a stage: BR, BS, S0, S1, S2, ALPHA; then the tile slots
    constexpr int OFF_BR = 0, OFF_BS = HS, OFF_S0 = 2 * HS, OFF_S1 = 3 * HS, OFF_S2 = 4 * HS,
                  OFF_AL = 5 * HS, OFF_T0 = 6 * HS;
    const float *stages = reinterpret_cast<const float *>(smem);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + NSTAGE * SB);

    if (tid == 0) {
        s_abort = 0;
        for (int i = 0; i < NSTAGE; ++i)
            mbar_init(&bars[i], 1);
        mbar_fence_init();
    }
    __syncthreads();

    // the thread's cells: rows r0-4+rho, r0-3+rho of the tile (box index rho)
    const int rho = G::TRW * w + C * lane;
    const int lane_row = C * lane;
    const bool rows_b = (lane_row >= 4 && lane_row < 60);   // B's output rows
    const bool producer = (tid == NT - 32);

    unsigned int q0 = 0;
    bool aborted = false;
    while (!aborted) {
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
        __syncthreads();
        if (item >= B.total_items)
            break;
        if (it < 0)
            continue;
        const ProblemDesc &P = B.probs[B.item_problem[item]];
        const int par = (it >> 1) & 1;   // one parity flip per pass
        const CUtensorMap *hmaps = P.halo[par];
        const CUtensorMap *tmaps = P.tile[par];
        const int nr = P.nr, ns = P.ns;
        const float cc = P.cc, inv_cc = P.inv_cc, steps = P.steps;
        const int li = item - P.item_begin;
        const int tile = li % P.tiles_r;
        const int chunk = li / P.tiles_r;
        const int s_begin = (int)((long long)ns * chunk / P.zchunks);
        const int s_end = (int)((long long)ns * (chunk + 1) / P.zchunks);
        const int r0 = tile * G::TR;
        const int n_steps = s_end - s_begin + 8;
        const int n_loads = n_steps + 1;
        const int p_first = s_begin - 4;
        float erru_a = 0.0f, erru_b = 0.0f;

        auto issue_load = [&](int j) {
            const unsigned int q = q0 + j;
            const int st = q % NSTAGE;
            const int plane = p_first + j;
            mbar_arrive_expect_tx(&bars[st], G::tx_bytes());
            float *base = const_cast<float *>(stages) + st * (SB / 4);
            tma_load_4d(base + OFF_BR, &hmaps[SL_BR], r0 - 4, 0, plane, 0, &bars[st]);
            tma_load_4d(base + OFF_BS, &hmaps[SL_BS], r0 - 4, 0, plane, 0, &bars[st]);
            tma_load_4d(base + OFF_S0, &hmaps[SL_S0], r0 - 4, 0, plane, 0, &bars[st]);
            tma_load_4d(base + OFF_S1, &hmaps[SL_S1], r0 - 4, 0, plane, 0, &bars[st]);
            tma_load_4d(base + OFF_S2, &hmaps[SL_S2], r0 - 4, 0, plane, 0, &bars[st]);
            tma_load_4d(base + OFF_AL, &hmaps[SL_ALPHA], r0 - 4, 0, plane, 0, &bars[st]);
#pragma unroll
            for (int ts = 0; ts < NUM_TILE_SLOTS; ++ts)
                tma_load_4d(base + OFF_T0 + ts * TS, &tmaps[ts], r0 - 4, 0, plane - 3, 0,
                            &bars[st]);
        };
        if (producer)
            for (int j = 0; j < NSTAGE && j < n_loads; ++j)
                issue_load(j);

        const int r = r0 - 4 + rho;
        bool inplane[C], fr_ok[C], fr1_ok[C];
        float fr_f[C], fr1_f[C];
#pragma unroll
        for (int j = 0; j < C; ++j) {
            const int rj = r + j;
            inplane[j] = (rj >= 0 && rj < nr);
            fr_ok[j] = (rj >= 1 && rj < nr);
            fr1_ok[j] = (rj + 1 >= 1 && rj + 1 < nr);
            fr_f[j] = fr_ok[j] ? 1.f : 0.f;
            fr1_f[j] = fr1_ok[j] ? 1.f : 0.f;
        }
        bool out_b[C];   // B's output cells of this thread
#pragma unroll
        for (int j = 0; j < C; ++j)
            out_b[j] = rows_b && inplane[j];
        const unsigned int col_off = (unsigned int)r;   // + plane * plane_stride
        const unsigned int plane_stride = (unsigned int)P.plane_stride;
        // halo-box reads rho .. rho+2, tile-box reads rho .. rho+1
        check_index(rho + 2, G::LR, P);
        check_index(rho + 1, G::TB, P);
        // B writes the pass's result into the other parity
        float *__restrict__ d_bs = P.dst_b[par][SL_BS];
        float *__restrict__ d_br = P.dst_b[par][SL_BR];
        float *__restrict__ d_s0 = P.dst_s[par][0];
        float *__restrict__ d_s1 = P.dst_s[par][1];
        float *__restrict__ d_s2 = P.dst_s[par][2];

        // carried state of iteration A (as in stencil2_kernel.cuh) ...
        float gkprev[C], bsprev[C], g2prev[C], alpha_prev[C];
        float br_prev[C], bss_cur[C], bss_old[C], dvp[C];
        // ... A's row faces r and r+1 of the previous step's plane, alpha two
        // and three planes back, A's pt/u and Cs/Ct of the last two epilogue
        // planes (B's epilogue runs two planes behind A's) ...
        float a_br[C], a_br1[C], alpha_d2[C], alpha_d3[C];
        float a_pt[2][C], a_u[2][C], c_cs[2][C], c_ct[2][C];
        // ... and of iteration B
        float gkprevB[C], bsprevB[C], g2prevB[C], br_prevB[C], bss_curB[C], bss_oldB[C], dvpB[C];
#pragma unroll
        for (int j = 0; j < C; ++j) {
            gkprev[j] = bsprev[j] = br_prev[j] = bss_cur[j] = bss_old[j] = dvp[j] = 0.f;
            g2prev[j] = 1.f;
            alpha_prev[j] = alpha_d2[j] = alpha_d3[j] = 1.f;
            a_br[j] = a_br1[j] = 0.f;
            a_pt[0][j] = a_pt[1][j] = a_u[0][j] = a_u[1][j] = 0.f;
            c_cs[0][j] = c_cs[1][j] = c_ct[0][j] = c_ct[1][j] = 0.f;
            gkprevB[j] = bsprevB[j] = br_prevB[j] = bss_curB[j] = bss_oldB[j] = dvpB[j] = 0.f;
            g2prevB[j] = 1.f;
        }

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

#pragma unroll UNROLL
        for (int t = 0; t < n_steps && !aborted; ++t) {
            const int s = p_first + t;
            const int st_cur = (q0 + t) % NSTAGE, st_nxt = (q0 + t + 1) % NSTAGE;
            bool wait_ok = true;
            if (t == 0)
                wait_ok = mbar_wait_bounded(&bars[st_cur], ((q0 + t) / NSTAGE) & 1, &s_abort);
            wait_ok = wait_ok && mbar_wait_bounded(&bars[st_nxt], ((q0 + t + 1) / NSTAGE) & 1,
                                                    &s_abort);
            const bool s_in = (s >= 0 && s < ns);
            const bool sb_in = (s >= 1 && s < ns);
            const bool sp_in = (s - 1 >= 0 && s - 1 < ns);
            const bool spb_in = (s - 1 >= 1 && s - 1 < ns);
            const bool sa_in = (s - 2 >= 0 && s - 2 < ns);   // A's epilogue plane
            const float sb_f = sb_in ? 1.f : 0.f, spb_f = spb_in ? 1.f : 0.f;

            // ---- A, X: gk(s) from the old state
            const float *Sc = stages + st_cur * (SB / 4) + rho;
            const float *Sn = stages + st_nxt * (SB / 4) + rho;
            float gk[C], by_own[C], bs_own[C], alpha_cur[C];
            {
                float d[C], v[C], s0[C], s1[C], s2[C];
                ld_cells<C>(Sc + OFF_BR, by_own);
                d[0] = by_own[1] - by_own[0];
                d[1] = Sc[OFF_BR + 2] - by_own[1];
                ld_cells<C>(Sc + OFF_BS, bs_own);
                ld_cells<C>(Sn + OFF_BS, v);
#pragma unroll
                for (int j = 0; j < C; ++j) {
                    d[j] = d[j] + v[j];
                    d[j] = d[j] - bs_own[j];
                }
                ld_cells<C>(Sc + OFF_S0, s0);
                ld_cells<C>(Sc + OFF_S1, s1);
                ld_cells<C>(Sc + OFF_S2, s2);
#pragma unroll
                for (int j = 0; j < C; ++j)
                    gk[j] = d[j] - ((s0[j] - s1[j]) + div_cc<EXACT>(s2[j], cc, inv_cc));
                ld_cells<C>(Sc + OFF_AL, alpha_cur);
            }
            // epilogue inputs of A (plane s-2, from the tile boxes of stage s+1)
            float t_pt[C], t_u[C], t_cs[C], t_ct[C];
            {
                const float *T = stages + st_nxt * (SB / 4) + OFF_T0 + rho;
                ld_cells<C>(T + TS_S1 * TS, t_pt);
                ld_cells<C>(T + TS_S2 * TS, t_u);
                ld_cells<C>(T + TS_CS * TS, t_cs);
                ld_cells<C>(T + TS_CT * TS, t_ct);
            }
            // Every thread has read what it needs of stage s: the slot can be
            // refilled once all have passed this barrier.
            if (__syncthreads_or(!wait_ok)) {
                aborted = true;
                abort_item(t, min(n_loads, t + NSTAGE));
                break;
            }
            if (producer && t + NSTAGE < n_loads)
                issue_load(t + NSTAGE);

            // ---- A, Y: b'(s), g2(s-1), b''_s(s-1)
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
            rows_down<C>(br_prev, br_dn);
#pragma unroll
            for (int j = 0; j < C; ++j)
                g2[j] = Proj<EXACT>::gk(bsn[j], bsprev[j], br_dn[j], br_prev[j], alpha_prev[j]);
#pragma unroll
            for (int j = 0; j < C; ++j) {
                bssn[j] = keep_if<EXACT>(((g2[j] + g2prev[j]) * 0.5f) * bsprev[j],
                                         inplane[j] && spb_in, spb_f);
                bss_old[j] = bss_cur[j];
                bss_cur[j] = bssn[j];
                g2prev[j] = g2[j];
                bsprev[j] = bsn[j];
            }

            // ---- A, Z: b''_r(s-1) (kept for B), ps/pt/u(s-2)
            float g2_up[C], g2_dn[C], brr[C], brr1[C], dn[C];
            rows_up<C>(g2, g2_up);
            rows_down<C>(g2, g2_dn);
#pragma unroll
            for (int j = 0; j < C; ++j) {
                brr[j] = keep_if<EXACT>(((g2[j] + g2_up[j]) * 0.5f) * br_prev[j], fr_ok[j] && sp_in,
                                        fr_f[j]);
                brr1[j] = keep_if<EXACT>(((g2_dn[j] + g2[j]) * 0.5f) * br_dn[j], fr1_ok[j] && sp_in,
                                         fr1_f[j]);
                dn[j] = brr1[j] - brr[j];
            }
            float ps_a[C], pt_a[C], u_a[C];
#pragma unroll
            for (int j = 0; j < C; ++j) {
                float dv = dvp[j] + bss_cur[j];
                dv = dv - bss_old[j];
                const float ucc = div_cc<EXACT>(t_u[j], cc, inv_cc);
                float ps_n = ((t_pt[j] - ucc) + dv) + inv_cc;
                ps_n = min_sel<EXACT>(ps_n, t_cs[j]);
                float pt_n = (ps_n + ucc) - dv;
                pt_n = min_sel<EXACT>(pt_n, t_ct[j]);
                const float e = cc * ((pt_n + dv) - ps_n);
                const bool live = inplane[j] && sa_in;   // outside the image the state is zero
                if (out_b[j] && s - 2 >= s_begin && s - 2 < s_end)
                    erru_a += abs_ref(e);
                ps_a[j] = live ? ps_n : 0.f;
                pt_a[j] = live ? pt_n : 0.f;
                u_a[j] = live ? t_u[j] - e : 0.f;
                dvp[j] = dn[j];
            }

            // ---- B, X at plane q = s-2 from A's results
            const int qp = s - 2;
            const bool q_in = (qp >= 0 && qp < ns);
            const bool qb_in = (qp >= 1 && qp < ns);
            const bool qp_in = (qp - 1 >= 0 && qp - 1 < ns);
            const bool qpb_in = (qp - 1 >= 1 && qp - 1 < ns);
            const float qb_f = qb_in ? 1.f : 0.f, qpb_f = qpb_in ? 1.f : 0.f;
            float gkB[C];
#pragma unroll
            for (int j = 0; j < C; ++j) {
                // A's row faces r and r+1 at plane q, stream faces q and q+1
                float d = a_br1[j] - a_br[j];
                d = d + bss_cur[j];
                d = d - bss_old[j];
                gkB[j] = d - ((ps_a[j] - pt_a[j]) + div_cc<EXACT>(u_a[j], cc, inv_cc));
            }
            // ---- B, Y: b'(q), g2(q-1), b''_s(q-1)
            float gk_upB[C], brnB[C], bsnB[C], br_dnB[C], g2B[C];
            rows_up<C>(gkB, gk_upB);
#pragma unroll
            for (int j = 0; j < C; ++j) {
                brnB[j] = keep_if<EXACT>(steps * (gkB[j] - gk_upB[j]) + a_br[j], fr_ok[j] && q_in,
                                         fr_f[j]);
                bsnB[j] = keep_if<EXACT>(steps * (gkB[j] - gkprevB[j]) + bss_old[j],
                                         inplane[j] && qb_in, qb_f);
                gkprevB[j] = gkB[j];
            }
            rows_down<C>(br_prevB, br_dnB);
#pragma unroll
            for (int j = 0; j < C; ++j)
                g2B[j] = Proj<EXACT>::gk(bsnB[j], bsprevB[j], br_dnB[j], br_prevB[j], alpha_d3[j]);
            {
                float bssnB[C];
#pragma unroll
                for (int j = 0; j < C; ++j)
                    bssnB[j] = keep_if<EXACT>(((g2B[j] + g2prevB[j]) * 0.5f) * bsprevB[j],
                                              inplane[j] && qpb_in, qpb_f);
                if (qp - 1 >= s_begin && qp - 1 < s_end)
                    st_dst<C>(d_bs, col_off + (unsigned int)(qp - 1) * plane_stride, bssnB, out_b,
                              P);
#pragma unroll
                for (int j = 0; j < C; ++j) {
                    bss_oldB[j] = bss_curB[j];
                    bss_curB[j] = bssnB[j];
                    g2prevB[j] = g2B[j];
                    bsprevB[j] = bsnB[j];
                }
            }
            // ---- B, Z: b''_r(q-1), the result at plane q-2
            {
                float g2_upB[C], g2_dnB[C], brrB[C], dnB[C];
                rows_up<C>(g2B, g2_upB);
                rows_down<C>(g2B, g2_dnB);
#pragma unroll
                for (int j = 0; j < C; ++j) {
                    brrB[j] = keep_if<EXACT>(((g2B[j] + g2_upB[j]) * 0.5f) * br_prevB[j],
                                             fr_ok[j] && qp_in, fr_f[j]);
                    const float brr1B = keep_if<EXACT>(((g2_dnB[j] + g2B[j]) * 0.5f) * br_dnB[j],
                                                       fr1_ok[j] && qp_in, fr1_f[j]);
                    dnB[j] = brr1B - brrB[j];
                }
                if (qp - 1 >= s_begin && qp - 1 < s_end)
                    st_dst<C>(d_br, col_off + (unsigned int)(qp - 1) * plane_stride, brrB, out_b, P);
                const int so = qp - 2;
                if (so >= s_begin && so < s_end) {
                    float ps_o[C], pt_o[C], u_o[C];
#pragma unroll
                    for (int j = 0; j < C; ++j) {
                        float dv = dvpB[j] + bss_curB[j];
                        dv = dv - bss_oldB[j];
                        const float ucc = div_cc<EXACT>(a_u[1][j], cc, inv_cc);
                        float ps_n = ((a_pt[1][j] - ucc) + dv) + inv_cc;
                        ps_n = min_sel<EXACT>(ps_n, c_cs[1][j]);
                        float pt_n = (ps_n + ucc) - dv;
                        pt_n = min_sel<EXACT>(pt_n, c_ct[1][j]);
                        const float e = cc * ((pt_n + dv) - ps_n);
                        if (out_b[j])
                            erru_b += abs_ref(e);
                        ps_o[j] = ps_n;
                        pt_o[j] = pt_n;
                        u_o[j] = a_u[1][j] - e;
                    }
                    const unsigned int o = col_off + (unsigned int)so * plane_stride;
                    st_dst<C>(d_s0, o, ps_o, out_b, P);
                    st_dst<C>(d_s1, o, pt_o, out_b, P);
                    st_dst<C>(d_s2, o, u_o, out_b, P);
                }
#pragma unroll
                for (int j = 0; j < C; ++j) {
                    dvpB[j] = dnB[j];
                    br_prevB[j] = brnB[j];
                }
            }

            // ---- shift the delay lines by one plane
#pragma unroll
            for (int j = 0; j < C; ++j) {
                br_prev[j] = brn[j];
                a_br[j] = brr[j];
                a_br1[j] = brr1[j];
                alpha_d3[j] = alpha_d2[j];
                alpha_d2[j] = alpha_prev[j];
                alpha_prev[j] = alpha_cur[j];
                a_pt[1][j] = a_pt[0][j];
                a_pt[0][j] = pt_a[j];
                a_u[1][j] = a_u[0][j];
                a_u[0][j] = u_a[j];
                c_cs[1][j] = c_cs[0][j];
                c_cs[0][j] = t_cs[j];
                c_ct[1][j] = c_ct[0][j];
                c_ct[0][j] = t_ct[j];
            }
            // the row shuffles of the next step read registers only; the stage
            // slots read this step are released by the next step's barrier
        }
        q0 += n_loads;
        __syncthreads();  // stage slots are reused by the next item
        finish_item_t2<NT>(erru_a, erru_b, P, li, it, B.done_count, s_red, &s_is_last);
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

}  // namespace asets
