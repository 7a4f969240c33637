// Fused ALM iteration kernel, column-per-thread form: one launch = one
// iteration of the continuous max-flow solver (all labels of a labelled
// model).
//
// It fuses, per label, the reference's updateP1, updatePX/PY/PZ, projStep,
// updateBX/BY/BZ and divergence sweeps (maxflow/asetsBinaryMF3D_mex.c:166-180)
// and, for the binary model, updateDIVPSPTU and the erriter sum (:398-437).
//
// Geometry.  Rows r (Matlab y, contiguous), columns c (Matlab x in 3D) and a
// stream axis s (z in 3D, x in 2D).  Each warp owns 32*CELLS consecutive
// rows: 32*CELLS - 4 tile rows plus two halo rows on each side.  In 3D warp
// w is column c0 - 2 + w of a (32*CELLS - 4) x (NW-4) tile; in 2D the NW
// warps are consecutive (32*CELLS - 4)-row sub-tiles.  Every thread owns
// CELLS adjacent rows (1 or 2) of one column for the whole sweep along s, so
// its indices, border flags and carried values stay in registers; row
// neighbours come from the thread itself or, for its first and last cell,
// through one warp shuffle, column neighbours through three small shared
// planes.  With two cells the shared-memory and global accesses are 8-byte
// pairs, and the per-step index, flag and barrier work is shared by both.  One iteration has a stencil radius of two cells, so
// step s computes
//   X: gk(s) = div b(s) - ((s0 - s1) + s2/cc)               all threads
//   Y: gradient step b'(s); projection g2(s-1); b''_s(s-1)   tile + 1
//   Z: b''_r, b''_c of plane s-1; ps/pt/u (or div) of s-2    tile
// with two block barriers per step.  Old-state planes come through a ring of
// 4D TMA tiled loads; a stage holds the halo boxes of its plane and, for the
// binary model, tile boxes of pt/u/Cs/Ct three planes behind: step t reads
// them from the stage of plane s+1 (the plane s-2 it writes), which stays
// resident until the next step's X.  Out-of-grid elements load as 0: the zero-flux
// border of the reference.
//
// Work split: each problem's (label, stream chunk, tile) items, ordered
// chunk-major so that blocks running at the same time hold neighbouring tiles
// at the same planes and share their halos through L2, are handed out by an
// atomic queue.  One launch serves several independent problems of one kind
// (a batch); each problem advances its own iteration when its last item
// finishes, and items of converged problems are skipped.
//
// Arithmetic follows the reference's float expressions (build flags:
// --fmad=false, IEEE div/sqrt).  EXACT forms |p| in double as projStep does;
// the fast path uses a float sum and the hardware reciprocal square root.
#pragma once

#include "device_common.cuh"
#include "iteration_end.cuh"
#include "kernel_args.h"

namespace asets {

template <int DIM, int NW, int CELLS = 1>
struct ColGeom {
    static_assert(DIM == 2 || DIM == 3, "2D or 3D");
    static_assert(CELLS == 1 || CELLS == 2, "one or two cells per thread");
    static constexpr int NT = 32 * NW;
    static constexpr int TRW = 32 * CELLS - 4;                // tile rows per warp
    static constexpr int TR = (DIM == 3) ? TRW : TRW * NW;    // tile rows
    static constexpr int TC = (DIM == 3) ? NW - 4 : 1;        // tile columns
    static_assert(DIM == 2 || NW >= 5, "3D needs at least one tile column");
    static constexpr int LR = TR + 8;                         // halo box rows (origin r0-4)
    static_assert(LR <= 256, "TMA box dimension limit");
    static constexpr int LC = (DIM == 3) ? TC + 4 : 1;        // halo box columns (origin c0-2)
    static constexpr int LC_BC = (DIM == 3) ? TC + 5 : 1;     // column-face box (+forward face)

    static constexpr int align128(int b) { return (b + 127) & ~127; }
    static constexpr int halo_floats(int slot) { return slot == SL_BC ? LR * LC_BC : LR * LC; }
    static constexpr int tile_floats() { return TR * TC; }
    static constexpr bool has_slot(int slot) { return !(DIM == 2 && slot == SL_BC); }
    template <int EPI>
    static constexpr int stage_bytes()
    {
        int b = 0;
        for (int s = 0; s < NUM_SLOTS; ++s)
            if (has_slot(s))
                b += align128(halo_floats(s) * 4);
        if (EPI == EPI_BINARY)
            b += NUM_TILE_SLOTS * align128(tile_floats() * 4);
        return b;
    }
    template <int EPI>
    static constexpr int tx_bytes()
    {
        int b = 0;
        for (int s = 0; s < NUM_SLOTS; ++s)
            if (has_slot(s))
                b += halo_floats(s) * 4;
        if (EPI == EPI_BINARY)
            b += NUM_TILE_SLOTS * tile_floats() * 4;
        return b;
    }
    static constexpr int plane_bytes() { return (DIM == 3) ? align128(NT * CELLS * 4) : 0; }
    template <int NSTAGE, int EPI>
    static constexpr int smem_bytes()
    {
        // stages | GK | BC | G2 | mbarriers | alignment slack
        return NSTAGE * stage_bytes<EPI>() + 3 * plane_bytes() + NSTAGE * 8 + 128;
    }
};

// CELLS consecutive floats (CELLS = 1 or 2, 8-byte aligned for 2) into v
template <int CELLS>
__device__ __forceinline__ void ld_cells(const float *p, float (&v)[CELLS])
{
    if constexpr (CELLS == 2) {
        const float2 t = *reinterpret_cast<const float2 *>(p);
        v[0] = t.x;
        v[1] = t.y;
    } else {
        v[0] = p[0];
    }
}
template <int CELLS>
__device__ __forceinline__ void st_cells(float *p, const float (&v)[CELLS])
{
    if constexpr (CELLS == 2)
        *reinterpret_cast<float2 *>(p) = make_float2(v[0], v[1]);
    else
        p[0] = v[0];
}
// global store of the cells whose flag is set; the flags of a pair are both
// set except past the last row (cell 1 alone out of range)
template <int CELLS>
__device__ __forceinline__ void st_cells_if(float *__restrict__ p, const float (&v)[CELLS],
                                            const bool (&ok)[CELLS])
{
    if constexpr (CELLS == 2) {
        if (ok[1])
            *reinterpret_cast<float2 *>(p) = make_float2(v[0], v[1]);
        else if (ok[0])
            p[0] = v[0];
    } else if (ok[0]) {
        p[0] = v[0];
    }
}
// st_cells_if at element offset `off` of a destination array of the
// problem.  The bounds-check build (-DASETS_BOUNDS_CHECK) first checks that
// every stored cell lies inside the array (P.dst_elems elements) and
// otherwise records DEV_ERR_BOUNDS and stores nothing.
template <int CELLS>
__device__ __forceinline__ void st_dst(float *__restrict__ base, unsigned int off,
                                       const float (&v)[CELLS], const bool (&ok)[CELLS],
                                       const ProblemDesc &P)
{
#ifdef ASETS_BOUNDS_CHECK
    int last = -1;
#pragma unroll
    for (int j = 0; j < CELLS; ++j)
        if (ok[j])
            last = j;
    if (last >= 0 && (long long)off + last >= P.dst_elems) {
        atomicOr(&P.ctl->error, DEV_ERR_BOUNDS);
        return;
    }
#endif
    st_cells_if<CELLS>(base + off, v, ok);
}

// Bounds-check build: record DEV_ERR_BOUNDS when a shared-memory index of
// the thread is outside [0, limit).
__device__ __forceinline__ void check_index(long long idx, long long limit, const ProblemDesc &P)
{
#ifdef ASETS_BOUNDS_CHECK
    if (idx < 0 || idx >= limit)
        atomicOr(&P.ctl->error, DEV_ERR_BOUNDS);
#else
    (void)idx;
    (void)limit;
    (void)P;
#endif
}

// value of the row above (r-1) / below (r+1) each cell: inside the thread,
// or through one warp shuffle for the first / last cell
template <int CELLS>
__device__ __forceinline__ void rows_up(const float (&v)[CELLS], float (&up)[CELLS])
{
    up[0] = __shfl_up_sync(0xffffffffu, v[CELLS - 1], 1);
#pragma unroll
    for (int j = 1; j < CELLS; ++j)
        up[j] = v[j - 1];
}
template <int CELLS>
__device__ __forceinline__ void rows_down(const float (&v)[CELLS], float (&dn)[CELLS])
{
#pragma unroll
    for (int j = 0; j + 1 < CELLS; ++j)
        dn[j] = v[j + 1];
    dn[CELLS - 1] = __shfl_down_sync(0xffffffffu, v[0], 1);
}

template <int NT>
__device__ __forceinline__ void finish_item(float erru, const ProblemDesc &P, int li, int it,
                                            unsigned int *done_count, double *s_red,
                                            int *s_is_last)
{
    // erriter of this item in double, then the last item of the problem's
    // iteration sums the item partials in item order (deterministic)
    const double part = block_sum_double<NT>(erru, s_red);
    IterControl *ctl = P.ctl;
    if (threadIdx.x == 0) {
        P.item_partials[li] = part;
        __threadfence();
        const unsigned int ticket = atomicAdd(&ctl->ticket, 1u);
        *s_is_last = (ticket == (unsigned int)P.n_items - 1);
    }
    __syncthreads();
    if (*s_is_last && threadIdx.x < 32) {
        __threadfence();
        double acc = 0.0;
        for (int b = threadIdx.x; b < P.n_items; b += 32)
            acc += __ldcg(P.item_partials + b);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) {
            // cvg[i] = total_err / (float)N, total_err a float
            // (maxflow/asetsBinaryMF3D_mex.c:183)
            const float c = __fdiv_rn((float)acc, ctl->denom);
            P.cvg[it] = c;
            ctl->last_iter = it;
            const bool conv = ctl->break_lt ? (c < ctl->err_bound) : (c <= ctl->err_bound);
            int done = 0;
            if (ctl->error || conv) {
                done = 1;
                ctl->it_num = it;
            } else if (it + 1 >= ctl->max_it) {
                done = 1;
                ctl->it_num = ctl->max_it;
            }
            ctl->ticket = 0;
            ctl->iter = it + 1;
            if (done) {
                ctl->done = 1;
                atomicAdd(done_count, 1u);
            }
            __threadfence();
        }
    }
    __syncthreads();
}

// LATE: the producer issues the refill at the start of Z instead of right
// after the X barrier.  In 3D its warp is a halo column, which has no
// epilogue work in Z, so the issue leaves the Y barrier's critical path.
template <int DIM, int NW, int NSTAGE, int EPI, bool EXACT, int MINB, int UNROLL = 1, int CELLS = 1,
          bool LATE = false>
__global__ void __launch_bounds__(32 * NW, MINB)
    stencil_col_kernel(const __grid_constant__ BatchArgs B)
{
    using G = ColGeom<DIM, NW, CELLS>;
    constexpr int NT = G::NT;
    constexpr int C = CELLS;
    static_assert(NSTAGE >= 4, "stage of plane s stays resident until step s ends");

    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ int s_abort;
    __shared__ double s_red[NT / 32];
    __shared__ int s_is_last;
    __shared__ int s_item;

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;

    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
    constexpr int SB = G::template stage_bytes<EPI>();
    auto halo_slot = [&](int st, int slot) -> float * {
        int off = st * SB;
        for (int s = 0; s < slot; ++s)
            if (G::has_slot(s))
                off += G::align128(G::halo_floats(s) * 4);
        return reinterpret_cast<float *>(smem + off);
    };
    auto tile_slot = [&](int st, int ts) -> float * {
        int off = st * SB;
        for (int s = 0; s < NUM_SLOTS; ++s)
            if (G::has_slot(s))
                off += G::align128(G::halo_floats(s) * 4);
        off += ts * G::align128(G::tile_floats() * 4);
        return reinterpret_cast<float *>(smem + off);
    };
    // float offsets of each slot inside a stage (compile-time constants)
    constexpr int OFF_BC = 0;
    constexpr int OFF_BR = OFF_BC + (G::has_slot(SL_BC) ? G::align128(G::halo_floats(SL_BC) * 4) / 4 : 0);
    constexpr int OFF_BS = OFF_BR + G::align128(G::halo_floats(SL_BR) * 4) / 4;
    constexpr int OFF_S0 = OFF_BS + G::align128(G::halo_floats(SL_BS) * 4) / 4;
    constexpr int OFF_S1 = OFF_S0 + G::align128(G::halo_floats(SL_S0) * 4) / 4;
    constexpr int OFF_S2 = OFF_S1 + G::align128(G::halo_floats(SL_S1) * 4) / 4;
    constexpr int OFF_AL = OFF_S2 + G::align128(G::halo_floats(SL_S2) * 4) / 4;
    constexpr int OFF_T0 = OFF_AL + G::align128(G::halo_floats(SL_ALPHA) * 4) / 4;
    constexpr int TSZ = G::align128(G::tile_floats() * 4) / 4;
    const float *stages = reinterpret_cast<const float *>(smem);
    float *planes = reinterpret_cast<float *>(smem + NSTAGE * SB);
    constexpr int PF = G::plane_bytes() / 4;
    // shared planes: gk, the column faces b'_c (one buffer: the neighbour's
    // previous face is read in X, before the barrier that precedes this
    // step's write in Y) and the projection factors g2
    float *GK = planes;
    float *BCp = planes + PF;
    float *G2p = planes + 2 * PF;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + NSTAGE * SB + 3 * G::plane_bytes());

    if (tid == 0) {
        s_abort = 0;
        for (int i = 0; i < NSTAGE; ++i)
            mbar_init(&bars[i], 1);
        mbar_fence_init();
    }
    __syncthreads();

    // per-thread constants; the thread's cells are rows rho .. rho+C-1 of
    // its warp's 32*C rows (two halo rows on each side)
    const int rho = (DIM == 3) ? C * lane : G::TRW * w + C * lane;   // first cell's row index
    const int si = rho + 2 + ((DIM == 3) ? w * G::LR : 0);            // halo box index
    const int gi = (lane + 32 * w) * C;                               // shared plane index (3D)
    const int gi_left = (w >= 1) ? gi - 32 * C : gi;                  // column c-1 (clamped)
    const int gi_right = (w + 1 < NW) ? gi + 32 * C : gi;             // column c+1 (clamped)
    const int lane_row = C * lane;                                    // row within the warp
    const bool tile_row = (lane_row >= 2 && lane_row < 32 * C - 2);
    const bool tile_col = (DIM == 3) ? (w >= 2 && w < G::TC + 2) : true;
    const int ti = (DIM == 3) ? (lane_row - 2) + (w - 2) * G::TRW : (rho - 2);
    // The thread that issues the TMA loads and waits on their barriers; the
    // other threads block in the following CTA barrier instead of polling.
    const bool producer = (tid == NT - 32);

    unsigned int q0 = 0;
    bool aborted = false;

    __shared__ int s_iter;
    while (!aborted) {
        // thread 0 takes the next item and reads its problem's iteration
        // state once for the whole block
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
        IterControl *ctl = P.ctl;
        const int par = it & 1;
        const CUtensorMap *hmaps = P.halo[par];
        const CUtensorMap *tmaps = P.tile[par];
        const int nr = P.nr, nc = P.nc, ns = P.ns;
        const float cc = P.cc, inv_cc = P.inv_cc, steps = P.steps;
        const int tiles = P.tiles_r * P.tiles_c;
        const int li = item - P.item_begin;
        // chunk-major order: neighbouring tiles of one chunk run together
        const int tile = li % tiles;
        const int rest = li / tiles;
        const int chunk = rest % P.zchunks;
        const int k = rest / P.zchunks;
        const int s_begin = (int)((long long)ns * chunk / P.zchunks);
        const int s_end = (int)((long long)ns * (chunk + 1) / P.zchunks);
        float erru = 0.0f;
        const int r0 = (tile % P.tiles_r) * G::TR;
        const int c0 = (DIM == 3) ? (tile / P.tiles_r) * G::TC : 0;
        const int n_steps = s_end - s_begin + 4;
        const int n_loads = n_steps + 1;
        const int p_first = s_begin - 2;
        const long long lab_off = (long long)k * P.label_stride;

        int lab_coord[NUM_SLOTS];
#pragma unroll
        for (int s = 0; s < NUM_SLOTS; ++s)
            lab_coord[s] = k * P.lab_mul[s] + P.lab_add[s];

        auto issue_load = [&](int j) {
            const unsigned int q = q0 + j;
            const int st = q % NSTAGE;
            const int plane = p_first + j;
            mbar_arrive_expect_tx(&bars[st], G::template tx_bytes<EPI>());
#pragma unroll
            for (int s = 0; s < NUM_SLOTS; ++s) {
                if (!G::has_slot(s))
                    continue;
                tma_load_4d(halo_slot(st, s), &hmaps[s], r0 - 4, (DIM == 3) ? c0 - 2 : 0, plane,
                            lab_coord[s], &bars[st]);
            }
            if constexpr (EPI == EPI_BINARY) {
#pragma unroll
                for (int ts = 0; ts < NUM_TILE_SLOTS; ++ts)
                    tma_load_4d(tile_slot(st, ts), &tmaps[ts], r0, c0, plane - 3, 0, &bars[st]);
            }
        };
        if (producer)
            for (int j = 0; j < NSTAGE && j < n_loads; ++j)
                issue_load(j);

        // this thread's cells (rows r .. r+C-1 of column c)
        const int r = r0 - 2 + rho;
        const int c = (DIM == 3) ? c0 - 2 + w : 0;
        const bool in_c = (c >= 0 && c < nc);
        bool inplane[C], is_tile[C], fr_ok[C], fr1_ok[C], fc_ok[C], fc1_ok[C];
        float fr_f[C], fr1_f[C], fc_f[C], fc1_f[C];
#pragma unroll
        for (int j = 0; j < C; ++j) {
            const int rj = r + j;
            const bool in_r = (rj >= 0 && rj < nr);
            inplane[j] = in_r && in_c;
            is_tile[j] = tile_row && tile_col && inplane[j];
            fr_ok[j] = (rj >= 1 && rj < nr && in_c);            // row face rj
            fr1_ok[j] = (rj + 1 >= 1 && rj + 1 < nr && in_c);   // row face rj+1
            fc_ok[j] = (in_r && c >= 1 && c < nc);
            fc1_ok[j] = (in_r && c + 1 >= 1 && c + 1 < nc);
            fr_f[j] = fr_ok[j] ? 1.f : 0.f;
            fr1_f[j] = fr1_ok[j] ? 1.f : 0.f;
            fc_f[j] = fc_ok[j] ? 1.f : 0.f;
            fc1_f[j] = fc1_ok[j] ? 1.f : 0.f;
        }
        // element offsets fit 32 bits: solves are limited to 2^31 - 1 voxel-labels
        const unsigned int col_off = (unsigned int)(lab_off + (long long)c * P.pitch + r);
        const unsigned int plane_stride = (unsigned int)P.plane_stride;
        // halo-box reads si .. si+C (the row face below the last cell), in 3D
        // the column faces of the next column si+LR .. si+LR+C-1; tile-box
        // reads ti .. ti+C-1; shared-plane reads gi .. gi+C-1
        check_index(si + C, G::LR * G::LC, P);
        if constexpr (DIM == 3)
            check_index(si + G::LR + C - 1, G::LR * G::LC_BC, P);
        if (is_tile[0])
            check_index(ti + C - 1, G::tile_floats(), P);
        if constexpr (DIM == 3)
            check_index(gi + C - 1, NT * C, P);
        float *__restrict__ d_bs = P.dst_b[par][SL_BS];
        float *__restrict__ d_br = P.dst_b[par][SL_BR];
        float *__restrict__ d_bc = P.dst_b[par][SL_BC];
        float *__restrict__ d_s0 = P.dst_s[par][0];
        float *__restrict__ d_s1 = P.dst_s[par][1];
        float *__restrict__ d_s2 = P.dst_s[par][2];

        float gkprev[C], bsprev[C], g2prev[C], alpha_prev[C];
        float br_prev[C], bc_prev[C], bss_cur[C], bss_old[C], dvp[C];
#pragma unroll
        for (int j = 0; j < C; ++j) {
            gkprev[j] = 0.f;
            bsprev[j] = 0.f;
            g2prev[j] = 1.f;
            alpha_prev[j] = 1.f;
            br_prev[j] = 0.f;
            bc_prev[j] = 0.f;
            bss_cur[j] = 0.f;
            bss_old[j] = 0.f;
            dvp[j] = 0.f;
        }

        // A wait gave up: drain this item's loads [first, issued) (bounded),
        // record the error and leave the item.
        auto abort_item = [&](int first, int issued) {
            if (producer) {
                s_abort = 0;
                for (int j = first; j < issued; ++j) {
                    const unsigned int q = q0 + j;
                    mbar_wait_bounded(&bars[q % NSTAGE], (q / NSTAGE) & 1, &s_abort);
                }
                atomicOr(&ctl->error, DEV_ERR_TIMEOUT);
            }
            __syncthreads();
        };
        // Step t reads the stages of planes t and t+1 (X; the binary Z also
        // reads the tile boxes of stage t+1), so after the X barrier no one
        // reads stage t any more and step t refills its slot with plane
        // t+NSTAGE.  Every thread waits for the stages it reads at the top of
        // the step that first reads them.  Two block barriers per step.
        constexpr int kLead = NSTAGE;   // refill the slot read by this X

#pragma unroll UNROLL
        for (int t = 0; t < n_steps && !aborted; ++t) {
            const int s = p_first + t;
            const int st_cur = (q0 + t) % NSTAGE, st_nxt = (q0 + t + 1) % NSTAGE;
            // Every thread waits on the mbarrier of the stage it is about to
            // read (stage t+1; stage t too on the first step), which also
            // makes the stage's data visible to it: no block barrier here, so
            // a warp starts X as soon as its data is there instead of after
            // the slowest warp's Z.  A timeout is acted on at the X barrier.
            bool wait_ok = true;
            if (t == 0)
                wait_ok = mbar_wait_bounded(&bars[st_cur], ((q0 + t) / NSTAGE) & 1, &s_abort);
            wait_ok = wait_ok && mbar_wait_bounded(&bars[st_nxt], ((q0 + t + 1) / NSTAGE) & 1, &s_abort);
            const bool s_in = (s >= 0 && s < ns);
            const bool sb_in = (s >= 1 && s < ns);          // stream face s is interior
            const bool sp_in = (s - 1 >= 0 && s - 1 < ns);
            const bool spb_in = (s - 1 >= 1 && s - 1 < ns);
            // Stream-face masks.  The fast path skips the plane masks of the
            // row and column faces and the in-volume factor of the stream
            // faces: outside the volume every state element loads as zero
            // and the border faces are stored as zero, so gk, b' and b'' of
            // such cells and planes come out zero anyway (EXACT keeps the
            // reference's selects).
            const float sb_f = sb_in ? 1.f : 0.f, spb_f = spb_in ? 1.f : 0.f;

            // ---- X: gk(s) from the old state
            const float *Sc = stages + st_cur * (SB / 4) + si;   // this column in stage s
            const float *Sn = stages + st_nxt * (SB / 4) + si;   // and in stage s+1
            float gk[C], by_own[C], bx_own[C], bs_own[C], alpha_cur[C], bc_rt[C];
            {
                float d[C], v[C];
                ld_cells<C>(Sc + OFF_BR, by_own);
                {
                    float nx[C];   // row faces r+1 .. r+C
                    if constexpr (C == 2) {
                        nx[0] = by_own[1];
                        nx[1] = Sc[OFF_BR + 2];
                    } else {
                        nx[0] = Sc[OFF_BR + 1];
                    }
#pragma unroll
                    for (int j = 0; j < C; ++j)
                        d[j] = nx[j] - by_own[j];
                }
                if constexpr (DIM == 3) {
                    ld_cells<C>(Sc + OFF_BC, bx_own);
                    ld_cells<C>(Sc + OFF_BC + G::LR, v);
#pragma unroll
                    for (int j = 0; j < C; ++j) {
                        d[j] = d[j] + v[j];
                        d[j] = d[j] - bx_own[j];
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < C; ++j)
                        bx_own[j] = 0.f;
                }
                ld_cells<C>(Sc + OFF_BS, bs_own);
                ld_cells<C>(Sn + OFF_BS, v);
#pragma unroll
                for (int j = 0; j < C; ++j) {
                    d[j] = d[j] + v[j];
                    d[j] = d[j] - bs_own[j];
                }
                float s0[C], s1[C], s2[C];
                ld_cells<C>(Sc + OFF_S0, s0);
                ld_cells<C>(Sc + OFF_S1, s1);
                ld_cells<C>(Sc + OFF_S2, s2);
#pragma unroll
                for (int j = 0; j < C; ++j)
                    gk[j] = d[j] - ((s0[j] - s1[j]) + div_cc<EXACT>(s2[j], cc, inv_cc));
                ld_cells<C>(Sc + OFF_AL, alpha_cur);
                if constexpr (DIM == 3) {
                    st_cells<C>(GK + gi, gk);
                    // b'_c(s-1) at c+1, written by the previous Y (before Y rewrites it)
                    ld_cells<C>(BCp + gi_right, bc_rt);
                }
            }
            if (__syncthreads_or(!wait_ok)) {
                aborted = true;
                // loads issued: the prologue, then one per earlier step
                abort_item(t, min(n_loads, t + NSTAGE));
                break;
            }

            // refill a slot whose last readers finished before the barrier
            if (!LATE && producer && t + kLead < n_loads)
                issue_load(t + kLead);

            // ---- Y: gradient step b'(s), projection g2(s-1), stream faces b''(s-1)
            float gk_up[C];
            rows_up<C>(gk, gk_up);
            float brn[C], bcn[C], bsn[C], br_dn[C], g2[C];
#pragma unroll
            for (int j = 0; j < C; ++j)
                brn[j] = keep_if<EXACT>(steps * (gk[j] - gk_up[j]) + by_own[j], fr_ok[j] && s_in,
                                        fr_f[j]);
            if constexpr (DIM == 3) {
                float gk_left[C];
                ld_cells<C>(GK + gi_left, gk_left);
#pragma unroll
                for (int j = 0; j < C; ++j)
                    bcn[j] = keep_if<EXACT>(steps * (gk[j] - gk_left[j]) + bx_own[j], fc_ok[j] && s_in,
                                            fc_f[j]);
                st_cells<C>(BCp + gi, bcn);
            } else {
#pragma unroll
                for (int j = 0; j < C; ++j)
                    bcn[j] = bc_rt[j] = 0.f;
            }
#pragma unroll
            for (int j = 0; j < C; ++j) {
                bsn[j] = keep_if<EXACT>(steps * (gk[j] - gkprev[j]) + bs_own[j], inplane[j] && sb_in, sb_f);
                gkprev[j] = gk[j];
            }
            rows_down<C>(br_prev, br_dn);   // b'_r(s-1) at r+1
#pragma unroll
            for (int j = 0; j < C; ++j) {
                if constexpr (DIM == 3)
                    g2[j] = Proj<EXACT>::gk(bc_rt[j], bc_prev[j], br_dn[j], br_prev[j], bsn[j], bsprev[j],
                                            alpha_prev[j]);
                else
                    g2[j] = Proj<EXACT>::gk(bsn[j], bsprev[j], br_dn[j], br_prev[j], alpha_prev[j]);
            }
            if constexpr (DIM == 3)
                st_cells<C>(G2p + gi, g2);
            const int sp = s - 1;
            {
                float bssn[C];
#pragma unroll
                for (int j = 0; j < C; ++j)
                    bssn[j] = keep_if<EXACT>(((g2[j] + g2prev[j]) * 0.5f) * bsprev[j],
                                             inplane[j] && spb_in, spb_f);
                if (sp >= s_begin && sp < s_end)
                    st_dst<C>(d_bs, col_off + (unsigned int)sp * plane_stride, bssn, is_tile, P);
#pragma unroll
                for (int j = 0; j < C; ++j) {
                    bss_old[j] = bss_cur[j];
                    bss_cur[j] = bssn[j];
                    g2prev[j] = g2[j];
                    bsprev[j] = bsn[j];
                    alpha_prev[j] = alpha_cur[j];
                }
            }
            __syncthreads();

            if (LATE && producer && t + kLead < n_loads)
                issue_load(t + kLead);

            // ---- Z: row/column faces of plane s-1 and the output of plane s-2
            {
                float g2_up[C], g2_dn[C], brr[C], dn[C], bcc[C];
                rows_up<C>(g2, g2_up);
                rows_down<C>(g2, g2_dn);
#pragma unroll
                for (int j = 0; j < C; ++j) {
                    brr[j] = keep_if<EXACT>(((g2[j] + g2_up[j]) * 0.5f) * br_prev[j], fr_ok[j] && sp_in,
                                            fr_f[j]);
                    const float brr1 = keep_if<EXACT>(((g2_dn[j] + g2[j]) * 0.5f) * br_dn[j],
                                                      fr1_ok[j] && sp_in, fr1_f[j]);
                    dn[j] = brr1 - brr[j];
                    bcc[j] = 0.f;
                }
                if constexpr (DIM == 3) {
                    float g2_l[C], g2_r[C];
                    ld_cells<C>(G2p + gi_left, g2_l);
                    ld_cells<C>(G2p + gi_right, g2_r);
#pragma unroll
                    for (int j = 0; j < C; ++j) {
                        bcc[j] = keep_if<EXACT>(((g2[j] + g2_l[j]) * 0.5f) * bc_prev[j], fc_ok[j] && sp_in,
                                                fc_f[j]);
                        const float bcc1 = keep_if<EXACT>(((g2_r[j] + g2[j]) * 0.5f) * bc_rt[j],
                                                          fc1_ok[j] && sp_in, fc1_f[j]);
                        dn[j] = dn[j] + bcc1;
                        dn[j] = dn[j] - bcc[j];
                    }
                }
                if (is_tile[0]) {
                    if (sp >= s_begin && sp < s_end) {
                        const unsigned int o = col_off + (unsigned int)sp * plane_stride;
                        st_dst<C>(d_br, o, brr, is_tile, P);
                        if constexpr (DIM == 3)
                            st_dst<C>(d_bc, o, bcc, is_tile, P);
                    }
                    const int so = s - 2;
                    if (so >= s_begin && so < s_end) {
                        float dv[C];
#pragma unroll
                        for (int j = 0; j < C; ++j) {
                            dv[j] = dvp[j] + bss_cur[j];
                            dv[j] = dv[j] - bss_old[j];
                        }
                        const unsigned int o = col_off + (unsigned int)so * plane_stride;
                        if constexpr (EPI == EPI_BINARY) {
                            const float *T = stages + st_nxt * (SB / 4) + OFF_T0 + ti;
                            float pt[C], u[C], csv[C], ctv[C], ps_o[C], pt_o[C], u_o[C];
                            ld_cells<C>(T + TS_S1 * TSZ, pt);
                            ld_cells<C>(T + TS_S2 * TSZ, u);
                            ld_cells<C>(T + TS_CS * TSZ, csv);
                            ld_cells<C>(T + TS_CT * TSZ, ctv);
#pragma unroll
                            for (int j = 0; j < C; ++j) {
                                const float ucc = div_cc<EXACT>(u[j], cc, inv_cc);
                                float ps_n = ((pt[j] - ucc) + dv[j]) + inv_cc;
                                ps_n = min_sel<EXACT>(ps_n, csv[j]);
                                float pt_n = (ps_n + ucc) - dv[j];
                                pt_n = min_sel<EXACT>(pt_n, ctv[j]);
                                const float e = cc * ((pt_n + dv[j]) - ps_n);
                                // cells past the last row hold zero state
                                // and add nothing
                                erru += abs_ref(e);
                                ps_o[j] = ps_n;
                                pt_o[j] = pt_n;
                                u_o[j] = u[j] - e;
                            }
                            st_dst<C>(d_s0, o, ps_o, is_tile, P);
                            st_dst<C>(d_s1, o, pt_o, is_tile, P);
                            st_dst<C>(d_s2, o, u_o, is_tile, P);
                        } else {
                            st_dst<C>(d_s0, o, dv, is_tile, P);
                        }
                    }
                }
#pragma unroll
                for (int j = 0; j < C; ++j) {
                    dvp[j] = dn[j];
                    br_prev[j] = brn[j];
                    bc_prev[j] = bcn[j];
                }
            }
        }
        q0 += n_loads;
        __syncthreads();  // stage slots and shared planes are reused by the next item
        if constexpr (EPI == EPI_BINARY)
            finish_item<NT>(erru, P, li, it, B.done_count, s_red, &s_is_last);
    }

    // the last block to leave re-arms the queue for the next launch
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
