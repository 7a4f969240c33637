// Argument blocks shared by the host runtime and the solver kernels.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace asets {

// Bits of IterControl::error.
enum DeviceError : int {
    DEV_ERR_TIMEOUT = 1,  // an mbarrier wait exceeded its budget
    DEV_ERR_BOUNDS = 2,   // bounds-check build: a store or shared-memory index out of range
};

// Per-solve control block in device memory.  Every iteration launch reads
// `done`/`iter` at entry; the last block of the iteration to finish (ticket)
// records erriter, decides convergence and advances `iter`.
struct IterControl {
    int iter;           // index of the next iteration
    int done;           // converged, maxIt reached, or error
    int it_num;         // the reference's itNum
    int last_iter;      // last executed iteration, -1 if none
    unsigned int ticket;
    int error;          // DeviceError bits
    int max_it;
    int break_lt;       // 1: stop on cvg < errBound (Ishikawa 2D), 0: on <=
    float err_bound;
    float denom;        // cvg = (float)erru / denom
    int alpha_bad;      // set by the validation pass
    int rollback;       // two-iteration pass: the solve ended at its first iteration
    int pad[4];
};

// Stage slots: which field each TMA box holds.
enum Slot : int {
    SL_BC = 0,   // flow on faces normal to the column axis (Matlab x in 3D)
    SL_BR = 1,   // flow on faces normal to the row axis (Matlab y)
    SL_BS = 2,   // flow on faces normal to the stream axis (z in 3D, x in 2D)
    SL_S0 = 3,   // gk source terms: gk = div - ((s0 - s1) + s2/cc)
    SL_S1 = 4,
    SL_S2 = 5,
    SL_ALPHA = 6,
    NUM_SLOTS = 7
};

enum Epilogue : int {
    EPI_BINARY = 0,  // binary model: ps/pt/u update + erriter
    EPI_DIV = 1,     // multi-label models: write the new flow and its divergence
    EPI_FUSED = 2,   // multi-label 2D, one pass: flows of all labels and the label update
};


// Arguments of the column-per-thread iteration kernel (stencil2_kernel.cuh).
// Halo slots are SL_BC..SL_ALPHA at the step's plane; tile slots carry the
// old pt and u and the capacities of the plane two steps behind (binary; the
// new ps needs no old ps).
enum TileSlot : int { TS_S1 = 0, TS_S2 = 1, TS_CS = 2, TS_CT = 3, NUM_TILE_SLOTS = 4 };

// One problem of a launch, in device memory (TMA descriptors need 64-byte
// alignment, which the CUtensorMap members give the struct).
struct ProblemDesc {
    CUtensorMap halo[2][NUM_SLOTS];        // [source parity][slot]
    CUtensorMap tile[2][NUM_TILE_SLOTS];   // binary; EPI_FUSED: [.][TS_CT] = Ct, all labels,
                                           // halo rows (the same map for both parities)
    float *dst_b[2][3];                    // [source parity][SL_BC, SL_BR, SL_BS]
    float *dst_s[2][3];                    // binary: ps, pt, u; EPI_DIV: [.][0] = divergence;
                                           // EPI_FUSED: Potts ps, pt, u; Ishikawa pt, -, u
    const float *alpha, *cs, *ct;          // inputs, for kernels that read them without TMA
    IterControl *ctl;
    double *item_partials;                 // binary: one erriter partial per item
    float *cvg;
    long long pitch;
    long long plane_stride;
    long long label_stride;
    int nr, nc, ns;
    int nlab_items;
    int tiles_r, tiles_c;
    int zchunks;                           // stream-axis chunks per tile
    int item_begin, n_items;               // this problem's items in the launch
    long long dst_elems;                   // elements of each destination array (bounds checks)
    int lab_mul[NUM_SLOTS];
    int lab_add[NUM_SLOTS];
    float cc, inv_cc, steps;
    float inv_cc_l;                        // EPI_FUSED Potts: 1/(cc*L), cc*L rounded to float
};

// A launch over one or more problems of the same kind (dimension, model).
struct BatchArgs {
    const ProblemDesc *probs;
    const int *item_problem;   // item -> problem index
    int total_items;
    unsigned int *queue;       // [0] next item, [1] blocks that left
    unsigned int *done_count;  // problems that have finished (shared by the launches of a batch)
};

}  // namespace asets
