// Binary 2D iteration on square tiles, for problems too small to keep the
// column sweep of stencil2_kernel.cuh busy.
//
// The sweep kernels walk each (tile, chunk) item plane by plane: on a 256^2
// image a launch has a few dozen items of 8-16 planes each, so the time of
// an iteration is the latency of one item's sweep, not bandwidth.  Here a
// block computes one whole iteration of an R x S tile (rows x stream
// columns) from the old state in phases over a shared frame of
// (R+5) x (S+5) cells (the tile and the iteration's two-cell halo, plus the
// faces beyond it): gk, then the gradient step b', the projection g2, the
// new flows b'' and, on the tile, the divergence and the ps/pt/u update with
// erriter -- the same float expressions, in the same order and with the
// same border masks, as the sweep kernel (EXACT results are bit-identical).
// Old state is read with coalesced loads through L2 (a small problem sits in
// L2), all of a thread's loads in flight at once; out-of-volume cells read
// as 0, the zero-flux border.  Two kernels: one launch per iteration, items
// handed out by the same queue and closed by the same per-item erriter
// partials and ticket as the sweeps; or every iteration in one cooperative
// launch with a grid barrier between iterations (every block resident, each
// taking one or more tiles), which removes the launch and hand-off latency
// that dominates an iteration of a small image.
#pragma once

#include "stencil2_kernel.cuh"

namespace asets {

template <int R, int S>
struct Tile2Geom {
    static constexpr int FR = R + 5;          // frame rows: r0-2 .. r0+R+2
    static constexpr int FC = S + 5;          // frame columns: s0-2 .. s0+S+2
    static constexpr int F = FR * FC;         // floats per frame array
    static constexpr int NARR = 10;           // BR BS PS PT U AL GK BR1 BS1 G2
    static constexpr int smem_bytes() { return NARR * F * 4 + 16; }
};

// One ALM iteration of tile li of problem P from parity par, in the frame
// `fsm` (Tile2Geom::NARR arrays): loads, the phases, the stores of the new
// flows and state.  Returns the thread's share of erriter.  State is read
// through L2 (ld.global.cg): the persistent kernel reads what other blocks
// wrote during the same launch.
template <int R, int S, int NT, bool EXACT>
__device__ __forceinline__ float tile2_iteration(const ProblemDesc &P, int par, int li, float *fsm)
{
    using G = Tile2Geom<R, S>;
    constexpr int FR = G::FR, F = G::F;
    float *BR = fsm, *BS = fsm + F, *PS = fsm + 2 * F, *PT = fsm + 3 * F, *U = fsm + 4 * F;
    float *AL = fsm + 5 * F, *GK = fsm + 6 * F, *BR1 = fsm + 7 * F, *BS1 = fsm + 8 * F;
    float *G2 = fsm + 9 * F;
    const int tid = threadIdx.x;
    const int nr = P.nr, ns = P.ns;
    const float cc = P.cc, inv_cc = P.inv_cc, steps = P.steps;
    const int r0 = (li % P.tiles_r) * R;
    const int s0 = (li / P.tiles_r) * S;
    const unsigned int pitch = (unsigned int)P.plane_stride;  // one row of Matlab x
    // old state: the other parity's destinations
    const float *src_br = P.dst_b[par ^ 1][SL_BR];
    const float *src_bs = P.dst_b[par ^ 1][SL_BS];
    const float *src_ps = P.dst_s[par ^ 1][0];
    const float *src_pt = P.dst_s[par ^ 1][1];
    const float *src_u = P.dst_s[par ^ 1][2];
        float erru = 0.0f;

        // Frame cell (c, q) <-> pixel (r0-2+q, s0-2+c).  Every load of the
        // thread (its frame cells, and Cs/Ct of its tile cells for the
        // update) is issued before the first is used: one memory round trip.
        constexpr int PER = (F + NT - 1) / NT;
        constexpr int PIX = (R * S + NT - 1) / NT;
        float v[6][PER], cs_v[PIX], ct_v[PIX];
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int i = tid + k * NT;
            const int c = i / FR, q = i - c * FR;
            const int r = r0 - 2 + q, s = s0 - 2 + c;
            const bool in = (i < F && r >= 0 && r < nr && s >= 0 && s < ns);
            const unsigned int g = (unsigned int)s * pitch + (unsigned int)r;
            v[0][k] = in ? __ldcg(src_br + g) : 0.f;
            v[1][k] = in ? __ldcg(src_bs + g) : 0.f;
            v[2][k] = in ? __ldcg(src_ps + g) : 0.f;
            v[3][k] = in ? __ldcg(src_pt + g) : 0.f;
            v[4][k] = in ? __ldcg(src_u + g) : 0.f;
            v[5][k] = in ? __ldcg(P.alpha + g) : 0.f;
        }
#pragma unroll
        for (int k = 0; k < PIX; ++k) {
            const int i = tid + k * NT;
            const int r = r0 + i % R, s = s0 + i / R;
            const bool in = (i < R * S && r < nr && s < ns);
            const unsigned int g = (unsigned int)s * pitch + (unsigned int)r;
            cs_v[k] = in ? __ldcg(P.cs + g) : 0.f;
            ct_v[k] = in ? __ldcg(P.ct + g) : 0.f;
        }
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int i = tid + k * NT;
            if (i < F) {
                BR[i] = v[0][k];
                BS[i] = v[1][k];
                PS[i] = v[2][k];
                PT[i] = v[3][k];
                U[i] = v[4][k];
                AL[i] = v[5][k];
            }
        }
        __syncthreads();

        // gk on rows r0-2 .. r0+R+1, columns s0-2 .. s0+S+1
        for (int i = tid; i < (R + 4) * (S + 4); i += NT) {
            const int c = i / (R + 4), q = i - c * (R + 4);
            const int f = c * FR + q;
            float d = BR[f + 1] - BR[f];
            d = d + BS[f + FR];
            d = d - BS[f];
            GK[f] = d - ((PS[f] - PT[f]) + div_cc<EXACT>(U[f], cc, inv_cc));
        }
        __syncthreads();

        // b'_r on faces r0-1 .. r0+R+1 of columns s0-1 .. s0+S; b'_s on
        // faces s0-1 .. s0+S+1 of rows r0-1 .. r0+R
        for (int i = tid; i < (R + 3) * (S + 2); i += NT) {
            const int c = 1 + i / (R + 3), q = 1 + i % (R + 3);
            const int f = c * FR + q;
            const int r = r0 - 2 + q, s = s0 - 2 + c;
            const bool fr_ok = (r >= 1 && r < nr), s_in = (s >= 0 && s < ns);
            BR1[f] = keep_if<EXACT>(steps * (GK[f] - GK[f - 1]) + BR[f], fr_ok && s_in,
                                    fr_ok ? 1.f : 0.f);
        }
        for (int i = tid; i < (R + 2) * (S + 3); i += NT) {
            const int c = 1 + i / (R + 2), q = 1 + i % (R + 2);
            const int f = c * FR + q;
            const int r = r0 - 2 + q, s = s0 - 2 + c;
            const bool inplane = (r >= 0 && r < nr), sb_in = (s >= 1 && s < ns);
            BS1[f] = keep_if<EXACT>(steps * (GK[f] - GK[f - FR]) + BS[f], inplane && sb_in,
                                    sb_in ? 1.f : 0.f);
        }
        __syncthreads();

        // g2 on rows r0-1 .. r0+R, columns s0-1 .. s0+S
        for (int i = tid; i < (R + 2) * (S + 2); i += NT) {
            const int c = 1 + i / (R + 2), q = 1 + i % (R + 2);
            const int f = c * FR + q;
            G2[f] = Proj<EXACT>::gk(BS1[f + FR], BS1[f], BR1[f + 1], BR1[f], AL[f]);
        }
        __syncthreads();

        // b''_r on faces r0 .. r0+R of the tile's columns, b''_s on faces
        // s0 .. s0+S of the tile's rows (into the old-flow arrays); the
        // tile's own faces are stored
        float *__restrict__ d_br = P.dst_b[par][SL_BR];
        float *__restrict__ d_bs = P.dst_b[par][SL_BS];
        for (int i = tid; i < (R + 1) * S; i += NT) {
            const int c = 2 + i / (R + 1), q = 2 + i % (R + 1);
            const int f = c * FR + q;
            const int r = r0 - 2 + q, s = s0 - 2 + c;
            const bool fr_ok = (r >= 1 && r < nr), sp_in = (s >= 0 && s < ns);
            const float v = keep_if<EXACT>(((G2[f] + G2[f - 1]) * 0.5f) * BR1[f], fr_ok && sp_in,
                                           fr_ok ? 1.f : 0.f);
            BR[f] = v;
            if (q < R + 2 && r < nr && s < ns)
                d_br[(unsigned int)s * pitch + (unsigned int)r] = v;
        }
        for (int i = tid; i < R * (S + 1); i += NT) {
            const int c = 2 + i / R, q = 2 + i % R;
            const int f = c * FR + q;
            const int r = r0 - 2 + q, s = s0 - 2 + c;
            const bool inplane = (r >= 0 && r < nr), spb_in = (s >= 1 && s < ns);
            const float v = keep_if<EXACT>(((G2[f] + G2[f - FR]) * 0.5f) * BS1[f],
                                           inplane && spb_in, spb_in ? 1.f : 0.f);
            BS[f] = v;
            if (c < S + 2 && r < nr && s < ns)
                d_bs[(unsigned int)s * pitch + (unsigned int)r] = v;
        }
        __syncthreads();

        // the tile: divergence of b'', ps/pt/u, erriter
        float *__restrict__ d_ps = P.dst_s[par][0];
        float *__restrict__ d_pt = P.dst_s[par][1];
        float *__restrict__ d_u = P.dst_s[par][2];
#pragma unroll
        for (int k = 0; k < PIX; ++k) {
            const int i = tid + k * NT;
            const int c = 2 + i / R, q = 2 + i % R;
            const int r = r0 - 2 + q, s = s0 - 2 + c;
            if (i >= R * S || r >= nr || s >= ns)
                continue;
            const int f = c * FR + q;
            float dv = BR[f + 1] - BR[f];
            dv = dv + BS[f + FR];
            dv = dv - BS[f];
            const unsigned int g = (unsigned int)s * pitch + (unsigned int)r;
            const float u = U[f];
            const float ucc = div_cc<EXACT>(u, cc, inv_cc);
            float ps_n = ((PT[f] - ucc) + dv) + inv_cc;
            ps_n = min_sel<EXACT>(ps_n, cs_v[k]);
            float pt_n = (ps_n + ucc) - dv;
            pt_n = min_sel<EXACT>(pt_n, ct_v[k]);
            const float e = cc * ((pt_n + dv) - ps_n);
            erru += abs_ref(e);
            d_ps[g] = ps_n;
            d_pt[g] = pt_n;
            d_u[g] = u - e;
        }
    __syncthreads();  // the frame is reused by the next item or iteration
    return erru;
}

template <int R, int S, int NT, bool EXACT, int MINB>
__global__ void __launch_bounds__(NT, MINB) stencil2d_tile_kernel(const __grid_constant__ BatchArgs B)
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
        const float erru = tile2_iteration<R, S, NT, EXACT>(P, it & 1, li, fsm);
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

// Every iteration of one problem in one cooperative launch: block b takes
// tiles b, b + grid, ... of every iteration (`iteration(it, tile)` returns
// the thread's erriter share); after each iteration the blocks meet at a grid barrier (an arrival
// counter, zeroed before the launch; each wait bounded by time, a timeout
// sets DEV_ERR_TIMEOUT and ends the solve), then every block sums the
// blocks' erriter partials in the order finish_item uses for items, so all
// take the same stopping decision; block 0 records cvg, itNum and the
// control block as finish_item does.  The launch and per-iteration hand-off of the
// one-launch-per-iteration form (queue, ticket, kernel boundary) is replaced
// by one barrier.  Partials alternate between two halves of item_partials by
// iteration parity.
template <int NT, class Iteration>
__device__ __forceinline__ void tile_solve_loop(const ProblemDesc &P, unsigned int *arrivals,
                                                double *s_red, int *s_stop, Iteration iteration)
{
    const int tid = threadIdx.x;
    IterControl *ctl = P.ctl;
    const int nb = (int)gridDim.x;   // at most one block per tile
    const int li = (int)blockIdx.x;
    if (*(volatile int *)&ctl->done)
        return;
    int it = *(volatile int *)&ctl->iter;
    const int max_it = ctl->max_it;
    const int break_lt = ctl->break_lt;
    const float err_bound = ctl->err_bound, denom = ctl->denom;
    for (unsigned int gen = 1;; ++gen) {
        float erru = 0.0f;
        for (int tile = li; tile < P.n_items; tile += nb)
            erru += iteration(it, tile);
        const double part = block_sum_double<NT>(erru, s_red);
        if (tid == 0) {
            P.item_partials[(it & 1) * nb + li] = part;
            __threadfence();
            atomicAdd(arrivals, 1u);
            // grid barrier: every block's state and partial of iteration it
            const unsigned int target = gen * (unsigned int)nb;
            int stop = 0;
            if (*(volatile unsigned int *)arrivals < target) {
                const unsigned long long t0 = global_timer_ns();
                while (*(volatile unsigned int *)arrivals < target) {
                    if (global_timer_ns() - t0 > kWaitBudgetNs) {
                        atomicOr(&ctl->error, DEV_ERR_TIMEOUT);
                        stop = 2;
                        break;
                    }
                }
            }
            __threadfence();
            *s_stop = stop;
        }
        __syncthreads();
        if (*s_stop == 2)
            break;  // a block did not arrive
        if (tid < 32) {
            double acc = 0.0;
            for (int b = tid; b < nb; b += 32)
                acc += __ldcg(P.item_partials + (it & 1) * nb + b);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (tid == 0) {
                // cvg[i] = total_err / (float)N, total_err a float (runMaxFlow)
                const float c = __fdiv_rn((float)acc, denom);
                const bool conv = break_lt ? (c < err_bound) : (c <= err_bound);
                const int done = (conv || it + 1 >= max_it) ? 1 : 0;
                if (li == 0) {
                    P.cvg[it] = c;
                    ctl->last_iter = it;
                    ctl->iter = it + 1;
                    if (done) {
                        ctl->it_num = conv ? it : max_it;
                        ctl->done = 1;
                    }
                    __threadfence();
                }
                *s_stop = done;
            }
        }
        __syncthreads();
        if (*s_stop)
            break;
        ++it;
    }
}

template <int R, int S, int NT, bool EXACT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
    stencil2d_tile_persistent_kernel(const __grid_constant__ BatchArgs B)
{
    extern __shared__ __align__(16) float fsm[];
    __shared__ double s_red[NT / 32];
    __shared__ int s_stop;
    const ProblemDesc &P = B.probs[0];
    tile_solve_loop<NT>(P, B.queue, s_red, &s_stop, [&](int it, int tile) {
        return tile2_iteration<R, S, NT, EXACT>(P, it & 1, tile, fsm);
    });
}

}  // namespace asets
