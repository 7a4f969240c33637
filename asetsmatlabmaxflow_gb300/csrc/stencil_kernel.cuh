// Fused ALM iteration kernel: one launch = one iteration of the continuous
// max-flow solver over the whole grid (all labels of a multi-label model).
//
// It fuses, per label, the reference's updateP1, updatePX/PY/PZ, projStep,
// updateBX/BY/BZ and divergence sweeps (maxflow/asetsBinaryMF3D_mex.c:166-180)
// into a single pass, and for the binary model also updateDIVPSPTU's
// source/sink/multiplier update and the erriter reduction (:398-437).
//
// Geometry.  The grid is viewed as rows r (Matlab y, contiguous), columns c
// (Matlab x in 3D; absent in 2D) and a stream axis s (z in 3D, x in 2D).  A
// block owns a TR x TC tile of (r, c) columns and marches along s over a
// range of planes.  One ALM iteration has a stencil radius of two cells, so
// each plane step needs the old state on the tile plus a 2-cell halo and
// produces new values with a lag of two planes:
//   step s:  gk(s)            on tile+2     (old state at s, s-faces at s+1)
//            b'(s)  faces     on tile+1/+2  (gradient step)
//            g2(s-1)          on tile+1     (projection factor)
//            b''(s-1) faces   on tile (+forward face)
//            ps/pt/u(s-2) or div(s-2) on the tile
// Old-state planes arrive through a ring of TMA tiled loads (zero-filled
// outside the grid, which is the reference's zero-flux border); the new
// state goes to the other buffer of a ping-pong pair.
//
// Arithmetic follows the reference's float expressions operation by
// operation (build flags: --fmad=false, IEEE div/sqrt); only |p| differs
// between EXACT (double, as projStep) and the fast path (float).
#pragma once

#include "device_common.cuh"
#include "iteration_end.cuh"
#include "kernel_args.h"

namespace asets {

template <int DIM, int TR, int TC>
struct TileGeom {
    static_assert(DIM == 2 || DIM == 3, "2D or 3D");
    static_assert(TR % 4 == 0, "TMA rows must start 16-byte aligned");
    static constexpr int LR = TR + 8;                   // TMA box rows, origin r0-4
    static_assert(LR <= 256, "TMA box dimension limit");
    static constexpr int GR = TR + 4;                   // region G rows, origin r0-2
    static constexpr int GC = (DIM == 3) ? TC + 4 : 1;  // region G cols, origin c0-2
    static constexpr int LC_BC = (DIM == 3) ? TC + 5 : 0;  // column-face box (+forward)
    static constexpr int LC = GC;                          // other boxes
    static constexpr int GP = GR * GC;                     // plane buffer (floats)
    static constexpr int R1R = TR + 2;                     // owner region (tile+1)
    static constexpr int R1C = (DIM == 3) ? TC + 2 : 1;
    static constexpr int R1 = R1R * R1C;
    static constexpr int FRR = TR + 3, FRC = (DIM == 3) ? TC + 2 : 1;   // row faces
    static constexpr int FCR = TR + 2, FCC = TC + 3;                    // column faces
    static constexpr int HRR = TR + 1, HRC = (DIM == 3) ? TC : 1;       // new row faces
    static constexpr int HCR = TR, HCC = TC + 1;                        // new col faces

    static constexpr int align128(int bytes) { return (bytes + 127) & ~127; }
    static constexpr int slot_floats(int slot)
    {
        return slot == SL_BC ? LR * LC_BC : LR * LC;
    }
    static constexpr int slot_bytes(int slot) { return align128(slot_floats(slot) * 4); }
    static constexpr int stage_bytes()
    {
        int b = 0;
        for (int s = 0; s < NUM_SLOTS; ++s)
            if (!(DIM == 2 && s == SL_BC))
                b += slot_bytes(s);
        return b;
    }
    static constexpr int tx_bytes()  // bytes one stage's TMA loads deliver
    {
        int b = 0;
        for (int s = 0; s < NUM_SLOTS; ++s)
            if (!(DIM == 2 && s == SL_BC))
                b += slot_floats(s) * 4;
        return b;
    }
    static constexpr int plane_bytes() { return align128(GP * 4); }
};

template <int DIM, int TR, int TC, int NSTAGE>
struct SmemLayout {
    using G = TileGeom<DIM, TR, TC>;
    static constexpr int kNumPlanes = 8;  // GK, BR x2, BC x2, G2, BRR, BCC
    static constexpr int stages = 0;
    static constexpr int planes = NSTAGE * G::stage_bytes();
    static constexpr int bars = planes + kNumPlanes * G::plane_bytes();
    static constexpr int total = bars + NSTAGE * 8 + 128;  // +128: base alignment
};

template <int DIM, int TR, int TC, int NT, int NSTAGE, int EPI, bool EXACT>
__global__ void __launch_bounds__(NT, (DIM == 3 ? 2 : 4))
    stencil_iteration_kernel(const __grid_constant__ StencilArgs A)
{
    using G = TileGeom<DIM, TR, TC>;
    using L = SmemLayout<DIM, TR, TC, NSTAGE>;
    constexpr int NSLOT = (G::R1 + NT - 1) / NT;
    static_assert(NSTAGE >= 3, "two planes resident plus one in flight");

    extern __shared__ __align__(128) unsigned char smem_raw[];
    // TMA destinations must be 128-byte aligned: align the carve-up base.
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
    __shared__ int s_abort;
    __shared__ double s_red[NT / 32];
    __shared__ int s_is_last;

    IterControl *ctl = A.ctl;
    if (*(volatile int *)&ctl->done)
        return;
    const int it = *(volatile int *)&ctl->iter;
    const int par = it & 1;
    const CUtensorMap *maps = A.map[par];
    const int tid = threadIdx.x;

    // ---- shared memory carve-up
    auto stage_slot = [&](int st, int slot) -> float * {
        int off = st * G::stage_bytes();
        for (int s = 0; s < slot; ++s)
            if (!(DIM == 2 && s == SL_BC))
                off += G::slot_bytes(s);
        return reinterpret_cast<float *>(smem + off);
    };
    float *planes = reinterpret_cast<float *>(smem + L::planes);
    constexpr int PF = G::plane_bytes() / 4;  // floats per plane buffer
    float *GK = planes;
    float *BRb[2] = {planes + 1 * PF, planes + 2 * PF};
    float *BCb[2] = {planes + 3 * PF, planes + 4 * PF};
    float *G2 = planes + 5 * PF;
    float *BRR = planes + 6 * PF;
    float *BCC = planes + 7 * PF;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L::bars);

    if (tid == 0) {
        s_abort = 0;
        for (int i = 0; i < NSTAGE; ++i)
            mbar_init(&bars[i], 1);
        mbar_fence_init();
        for (int s = 0; s < NUM_SLOTS; ++s)
            if (!(DIM == 2 && s == SL_BC))
                tma_prefetch_desc(&maps[s]);
    }
    __syncthreads();

    const int nr = A.nr, nc = A.nc, ns = A.ns;
    const float cc = A.cc, inv_cc = A.inv_cc, steps = A.steps;
    const int tiles = A.tiles_r * A.tiles_c;
    const long long total = A.total_work;
    const long long w0 = total * blockIdx.x / gridDim.x;
    const long long w1 = total * (blockIdx.x + 1) / gridDim.x;

    float erru = 0.0f;
    unsigned int q0 = 0;   // TMA load sequence number (phase bookkeeping)
    bool aborted = false;

    for (long long lin = w0; lin < w1 && !aborted;) {
        const long long item = lin / ns;
        const int s_begin = (int)(lin % ns);
        const int s_end = (int)((long long)s_begin + (w1 - lin) < ns ? s_begin + (w1 - lin) : ns);
        lin += s_end - s_begin;
        const int k = (int)(item / tiles);
        const int tile = (int)(item % tiles);
        const int r0 = (tile % A.tiles_r) * TR;
        const int c0 = (DIM == 3) ? (tile / A.tiles_r) * TC : 0;
        const int n_steps = s_end - s_begin + 4;
        const int n_loads = n_steps + 1;
        const int p_first = s_begin - 2;  // plane of load 0
        const long long lab_off = (long long)k * A.label_stride;

        int lab_coord[NUM_SLOTS];
#pragma unroll
        for (int s = 0; s < NUM_SLOTS; ++s)
            lab_coord[s] = k * A.lab_mul[s] + A.lab_add[s];

        auto issue_load = [&](int j) {  // load plane p_first + j into its slot
            const unsigned int q = q0 + j;
            const int st = q % NSTAGE;
            mbar_arrive_expect_tx(&bars[st], G::tx_bytes());
            const int plane = p_first + j;
#pragma unroll
            for (int s = 0; s < NUM_SLOTS; ++s) {
                if (DIM == 2 && s == SL_BC)
                    continue;
                tma_load_4d(stage_slot(st, s), &maps[s], r0 - 4, (DIM == 3) ? c0 - 2 : 0, plane,
                            lab_coord[s], &bars[st]);
            }
        };
        if (tid == 0)
            for (int j = 0; j < NSTAGE && j < n_loads; ++j)
                issue_load(j);

        // per-owner-cell carried state (owner region = tile + 1 ring)
        float gkprev[NSLOT], bsprev[NSLOT], g2prev[NSLOT], alphaprev[NSLOT];
        float bss_cur[NSLOT], bss_old[NSLOT], dvp[NSLOT];
        float qa0[NSLOT], qa1[NSLOT], qa2[NSLOT], qb0[NSLOT], qb1[NSLOT], qb2[NSLOT];
        float csa[NSLOT], cta[NSLOT];
#pragma unroll
        for (int j = 0; j < NSLOT; ++j) {
            gkprev[j] = 0.f; bsprev[j] = 0.f; g2prev[j] = 1.f; alphaprev[j] = 1.f;
            bss_cur[j] = 0.f; bss_old[j] = 0.f; dvp[j] = 0.f;
            qa0[j] = qa1[j] = qa2[j] = qb0[j] = qb1[j] = qb2[j] = 0.f;
            csa[j] = cta[j] = 0.f;
        }

        for (int t = 0; t < n_steps; ++t) {
            const int s = p_first + t;  // plane of this step's gk
            if (tid == 0 && t >= 1 && t + NSTAGE - 1 < n_loads)
                issue_load(t + NSTAGE - 1);
            const int st_cur = (q0 + t) % NSTAGE, st_nxt = (q0 + t + 1) % NSTAGE;
            bool ok = mbar_wait_bounded(&bars[st_cur], ((q0 + t) / NSTAGE) & 1, &s_abort);
            ok = ok && mbar_wait_bounded(&bars[st_nxt], ((q0 + t + 1) / NSTAGE) & 1, &s_abort);
            if (__syncthreads_or(!ok)) {
                aborted = true;
                // drain the loads still in flight (bounded), then leave
                if (tid == 0) {
                    s_abort = 0;
                    const int issued = min(n_loads, t + NSTAGE);
                    for (int j = t; j < issued; ++j) {
                        unsigned int q = q0 + j;
                        mbar_wait_bounded(&bars[q % NSTAGE], (q / NSTAGE) & 1, &s_abort);
                    }
                    atomicOr(&ctl->error, DEV_ERR_TIMEOUT);
                }
                __syncthreads();
                break;
            }
            const float *S_bc = stage_slot(st_cur, SL_BC);
            const float *S_br = stage_slot(st_cur, SL_BR);
            const float *S_bs = stage_slot(st_cur, SL_BS);
            const float *S_bs_next = stage_slot(st_nxt, SL_BS);
            const float *S_s0 = stage_slot(st_cur, SL_S0);
            const float *S_s1 = stage_slot(st_cur, SL_S1);
            const float *S_s2 = stage_slot(st_cur, SL_S2);
            const float *S_al = stage_slot(st_cur, SL_ALPHA);
            const bool s_in = (s >= 0 && s < ns);
            const int pb_cur = t & 1, pb_prev = pb_cur ^ 1;
            float *BRc = BRb[pb_cur], *BCc = BCb[pb_cur];
            const float *BRp = BRb[pb_prev], *BCp = BCb[pb_prev];

            // ---- P1: gk(s) = div b(s) - ((s0 - s1) + s2/cc) on tile + 2
            for (int i = tid; i < G::GP; i += NT) {
                const int gr = i % G::GR, gc = i / G::GR;
                const int si = gr + 2 + gc * G::LR;
                float d = S_br[si + 1] - S_br[si];
                if constexpr (DIM == 3) {
                    d = d + S_bc[si + G::LR];
                    d = d - S_bc[si];
                }
                d = d + S_bs_next[si];
                d = d - S_bs[si];
                GK[i] = d - ((S_s0[si] - S_s1[si]) + __fdiv_rn(S_s2[si], cc));
            }
            __syncthreads();

            // ---- P2a: gradient step on row faces (and column faces in 3D)
            for (int i = tid; i < G::FRR * G::FRC; i += NT) {
                const int gr = 1 + i % G::FRR;
                const int gc = (DIM == 3) ? 1 + i / G::FRR : 0;
                const int r = r0 - 2 + gr, c = (DIM == 3) ? c0 - 2 + gc : 0;
                const int gi = gr + gc * G::GR;
                float v = 0.f;
                if (r >= 1 && r < nr && c >= 0 && c < nc && s_in)
                    v = steps * (GK[gi] - GK[gi - 1]) + S_br[gr + 2 + gc * G::LR];
                BRc[gi] = v;
            }
            if constexpr (DIM == 3) {
                for (int i = tid; i < G::FCR * G::FCC; i += NT) {
                    const int gr = 1 + i % G::FCR, gc = 1 + i / G::FCR;
                    const int r = r0 - 2 + gr, c = (DIM == 3) ? c0 - 2 + gc : 0;
                    const int gi = gr + gc * G::GR;
                    float v = 0.f;
                    if (r >= 0 && r < nr && c >= 1 && c < nc && s_in)
                        v = steps * (GK[gi] - GK[gi - G::GR]) + S_bc[gr + 2 + gc * G::LR];
                    BCc[gi] = v;
                }
            }

            // ---- P2b: stream faces b'(s), projection g2(s-1), b''_s(s-1)
            const int sp = s - 1;  // plane of g2 / b'' this step
            const bool sp_out = (sp >= s_begin && sp < s_end);
#pragma unroll
            for (int j = 0; j < NSLOT; ++j) {
                const int i = tid + j * NT;
                if (i < G::R1) {
                    const int gr = 1 + i % G::R1R;
                    const int gc = (DIM == 3) ? 1 + i / G::R1R : 0;
                    const int r = r0 - 2 + gr, c = (DIM == 3) ? c0 - 2 + gc : 0;
                    const int gi = gr + gc * G::GR, si = gr + 2 + gc * G::LR;
                    const bool inplane = (r >= 0 && r < nr && c >= 0 && c < nc);
                    const float gk_now = GK[gi];
                    float bsp = 0.f;
                    if (inplane && s >= 1 && s < ns)
                        bsp = steps * (gk_now - gkprev[j]) + S_bs[si];
                    gkprev[j] = gk_now;
                    float g2;
                    if constexpr (DIM == 3)
                        g2 = Proj<EXACT>::gk(BCp[gi + G::GR], BCp[gi], BRp[gi + 1], BRp[gi], bsp,
                                             bsprev[j], alphaprev[j]);
                    else
                        g2 = Proj<EXACT>::gk(bsp, bsprev[j], BRp[gi + 1], BRp[gi], alphaprev[j]);
                    G2[gi] = g2;
                    float bss = 0.f;
                    if (inplane && sp >= 1 && sp < ns)
                        bss = ((g2 + g2prev[j]) * 0.5f) * bsprev[j];
                    const bool tile_cell = (gr >= 2 && gr < TR + 2 && gc >= (DIM == 3 ? 2 : 0) &&
                                            gc < (DIM == 3 ? TC + 2 : 1));
                    if (tile_cell && inplane && sp_out)
                        A.dst_b[par][SL_BS][lab_off + (long long)sp * A.plane_stride +
                                            (long long)c * A.pitch + r] = bss;
                    bss_old[j] = bss_cur[j];
                    bss_cur[j] = bss;
                    g2prev[j] = g2;
                    bsprev[j] = bsp;
                    alphaprev[j] = S_al[si];
                }
            }
            __syncthreads();

            // ---- P3: rescale row/column faces of plane s-1
            const bool sp_in = (sp >= 0 && sp < ns);
            for (int i = tid; i < G::HRR * G::HRC; i += NT) {
                const int gr = 2 + i % G::HRR;
                const int gc = (DIM == 3) ? 2 + i / G::HRR : 0;
                const int r = r0 - 2 + gr, c = (DIM == 3) ? c0 - 2 + gc : 0;
                const int gi = gr + gc * G::GR;
                float v = 0.f;
                if (r >= 1 && r < nr && c >= 0 && c < nc && sp_in)
                    v = ((G2[gi] + G2[gi - 1]) * 0.5f) * BRp[gi];
                BRR[gi] = v;
                if (gr < TR + 2 && r < nr && c < nc && sp_out)
                    A.dst_b[par][SL_BR][lab_off + (long long)sp * A.plane_stride +
                                        (long long)c * A.pitch + r] = v;
            }
            if constexpr (DIM == 3) {
                for (int i = tid; i < G::HCR * G::HCC; i += NT) {
                    const int gr = 2 + i % G::HCR, gc = 2 + i / G::HCR;
                    const int r = r0 - 2 + gr, c = (DIM == 3) ? c0 - 2 + gc : 0;
                    const int gi = gr + gc * G::GR;
                    float v = 0.f;
                    if (r >= 0 && r < nr && c >= 1 && c < nc && sp_in)
                        v = ((G2[gi] + G2[gi - G::GR]) * 0.5f) * BCp[gi];
                    BCC[gi] = v;
                    if (gc < TC + 2 && r < nr && c < nc && sp_out)
                        A.dst_b[par][SL_BC][lab_off + (long long)sp * A.plane_stride +
                                            (long long)c * A.pitch + r] = v;
                }
            }
            __syncthreads();

            // ---- P4: divergence of plane s-1's new faces; output plane s-2
            const int so = s - 2;
            const bool so_out = (so >= s_begin && so < s_end);
#pragma unroll
            for (int j = 0; j < NSLOT; ++j) {
                const int i = tid + j * NT;
                if (i < G::R1) {
                    const int gr = 1 + i % G::R1R;
                    const int gc = (DIM == 3) ? 1 + i / G::R1R : 0;
                    const bool tile_cell = (gr >= 2 && gr < TR + 2 &&
                                            gc >= (DIM == 3 ? 2 : 0) && gc < (DIM == 3 ? TC + 2 : 1));
                    if (tile_cell) {
                        const int r = r0 - 2 + gr, c = (DIM == 3) ? c0 - 2 + gc : 0;
                        const int gi = gr + gc * G::GR, si = gr + 2 + gc * G::LR;
                        const bool inplane = (r < nr && c < nc);
                        float dn = BRR[gi + 1] - BRR[gi];
                        if constexpr (DIM == 3) {
                            dn = dn + BCC[gi + G::GR];
                            dn = dn - BCC[gi];
                        }
                        if (inplane && so_out) {
                            float dv = dvp[j] + bss_cur[j];
                            dv = dv - bss_old[j];
                            const long long o = lab_off + (long long)so * A.plane_stride +
                                                (long long)c * A.pitch + r;
                            if constexpr (EPI == EPI_BINARY) {
                                const float u = qa2[j], pt = qa1[j];
                                const float ucc = __fdiv_rn(u, cc);
                                float ps_n = ((pt - ucc) + dv) + inv_cc;
                                ps_n = min_ref(ps_n, csa[j]);
                                float pt_n = (ps_n + ucc) - dv;
                                pt_n = min_ref(pt_n, cta[j]);
                                const float e = cc * ((pt_n + dv) - ps_n);
                                erru += abs_ref(e);
                                A.dst_s[par][0][o] = ps_n;
                                A.dst_s[par][1][o] = pt_n;
                                A.dst_s[par][2][o] = u - e;
                            } else {
                                A.dst_s[par][0][o] = dv;
                            }
                        }
                        dvp[j] = dn;
                        if constexpr (EPI == EPI_BINARY) {
                            qa0[j] = qb0[j]; qa1[j] = qb1[j]; qa2[j] = qb2[j];
                            qb0[j] = S_s0[si]; qb1[j] = S_s1[si]; qb2[j] = S_s2[si];
                            // capacities of plane s-1, consumed next step
                            const int sn = s - 1;
                            if (inplane && sn >= s_begin && sn < s_end) {
                                const long long on = (long long)sn * A.plane_stride +
                                                     (long long)c * A.pitch + r;
                                csa[j] = __ldg(A.cs + on);
                                cta[j] = __ldg(A.ct + on);
                            }
                        }
                    }
                }
            }
            __syncthreads();
        }
        q0 += n_loads;
    }

    if constexpr (EPI == EPI_BINARY)
        finish_iteration<NT>(erru, ctl, A.partials, A.cvg, it, s_red, &s_is_last);
}

}  // namespace asets
