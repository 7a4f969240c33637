// Internal interfaces between the host runtime and the kernel translation
// units of libasetscuda.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "kernel_args.h"

struct asets_context;

namespace asets {

// ---------------------------------------------------------------- stencil
// Label extent of the TMA boxes: one label (the label is the item's), or
// all labels of the array (stencil2d_labels_kernel).
enum LabelBoxes : int { LB_ONE = 0, LB_ALL = 1 };

// One compiled instance of an iteration kernel.
struct StencilVariant {
    int dim, epi, exact;
    int tr, tc, nt, nstage;  // tile rows/cols, threads, TMA ring depth
    int smem_bytes;          // dynamic shared memory per block
    int box_rows;            // halo box rows (tr + 8; tr + 12 for two iterations per pass)
    int box_cols;            // halo box columns for slots other than SL_BC
    int box_cols_bc;         // halo box columns of the SL_BC slot
    int tile_box_rows;       // rows of the binary tile boxes (tr; tr + 8 from row r0-4
                             // for two iterations per pass)
    int temporal;            // ALM iterations per launch (1, or 2: stencil2d_t2.cuh)
    const void *fn;
    int label_boxes = LB_ONE;
    int ct_box_rows = 0;     // rows of the Ct box of the one-pass multi-label kernel (0: none)
    int s_tile = 0;          // stream columns of a square-tile kernel's tile (0: a sweep)
    int persistent = 0;      // 1: every iteration in one cooperative launch, one block per tile
    // dynamic shared memory of a launch: smem_bytes + smem_per_fl x flow
    // labels + smem_per_l x labels (label counts known only at run time)
    int smem_per_fl = 0, smem_per_l = 0;
};

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Device buffers of one problem in the padded layout, as the iteration
// kernel sees them.
struct StencilProblem {
    int nr, nc, ns;              // rows, columns (1 in 2D), stream length
    long long pitch, plane, cells;
    int flow_labels;             // labels swept per launch
    float *b[2][3];              // flows [parity][SL_BC, SL_BR, SL_BS]
    float *src[2][3];            // gk sources s0, s1, s2 per parity
    int src_labels[3];           // label extent of each source array
    int lab_mul[NUM_SLOTS], lab_add[NUM_SLOTS];
    float *alpha;
    int alpha_labels;
    const float *cs, *ct;        // binary capacities; Ct of the one-pass multi-label kernel
    int ct_labels;
    float *dst_s[2][3];          // binary: new ps/pt/u; labelled: [.][0] = divergence
};

// Fill the TMA descriptors, destinations and geometry of problem `d` for
// variant `v` (ctl/cvg/item_partials/items/cc are set by the caller).
// Returns 0, or the CUresult of a failed encode.
int build_problem_desc(EncodeTiledFn encode, const StencilVariant &v, const StencilProblem &p,
                       ProblemDesc *d);
// Work split: stream-axis chunks per tile for `slots` resident blocks.
int choose_zchunks(const StencilProblem &p, const StencilVariant &v, long long slots);
// Items of one problem with the given chunk count.
int problem_items(const StencilProblem &p, const StencilVariant &v, int zchunks);

// Variant tables, one per translation unit.
const StencilVariant *binary3d_fast_variants(int *count);
const StencilVariant *binary3d_exact_variants(int *count);
const StencilVariant *binary2d_fast_variants(int *count);
const StencilVariant *binary2d_exact_variants(int *count);
const StencilVariant *flow3d_fast_variants(int *count);
const StencilVariant *flow3d_exact_variants(int *count);
const StencilVariant *flow2d_fast_variants(int *count);
const StencilVariant *flow2d_exact_variants(int *count);
// The compiled variants of one kind (dimension, epilogue, EXACT or fast);
// tile_config k >= 1 selects entry k-1.
inline const StencilVariant *stencil_variants(int dim, int epi, int exact, int *count)
{
    if (dim == 3)
        return epi == EPI_BINARY ? (exact ? binary3d_exact_variants(count) : binary3d_fast_variants(count))
                                 : (exact ? flow3d_exact_variants(count) : flow3d_fast_variants(count));
    return epi == EPI_BINARY ? (exact ? binary2d_exact_variants(count) : binary2d_fast_variants(count))
                             : (exact ? flow2d_exact_variants(count) : flow2d_fast_variants(count));
}

// The one-pass multi-label 2D kernels (stencil2d_labels.cuh) for a label
// count: Potts 1-8 labels, Ishikawa 2-9; `which` numbers the kernels of one
// label count from 0 (null past the last, or outside the range).
const StencilVariant *potts2d_fused_fast_variant(int nlab, int which);
const StencilVariant *potts2d_fused_exact_variant(int nlab, int which);
const StencilVariant *ishikawa2d_fused_fast_variant(int nlab, int which);
const StencilVariant *ishikawa2d_fused_exact_variant(int nlab, int which);
// model: 1 Potts, 2 Ishikawa
inline const StencilVariant *fused2d_variant(int model, int nlab, int exact, int which = 0)
{
    if (model == 1)
        return exact ? potts2d_fused_exact_variant(nlab, which) : potts2d_fused_fast_variant(nlab, which);
    if (model == 2)
        return exact ? ishikawa2d_fused_exact_variant(nlab, which)
                     : ishikawa2d_fused_fast_variant(nlab, which);
    return nullptr;
}

// ---------------------------------------------------------------- labels
struct LabelArgs {
    float *u;
    float *pt;
    float *ps;           // Potts only
    const float *dv;
    const float *ct;
    IterControl *ctl;
    double *partials;
    float *cvg;
    long long cells;         // padded cells per label
    long long label_stride;  // == cells
    unsigned int rows;       // padded rows per label (cells / pitch)
    int pitch, nr, nlab;
    float cc, inv_cc, inv_cc_l;  // 1/cc and 1/(cc*L) as the reference rounds them
    int exact;               // 1: the reference's divisions; 0: reciprocal multiplies
    unsigned int *done_count;  // batch: finished-problem counter, or null
};

int label_kernel_grid(long long cells, int num_sms);
cudaError_t launch_potts_labels(const LabelArgs &a, int grid, cudaStream_t st);
cudaError_t launch_ishikawa_labels(const LabelArgs &a, int grid, cudaStream_t st);

// ---------------------------------------------------------------- init
struct InitArgs {
    const float *cs;
    const float *ct;
    const float *alpha;
    float *u, *ps, *pt;
    IterControl *ctl;
    long long cells;         // padded cells per label
    long long label_stride;
    int pitch, nr, nlab;
    int alpha_labels;        // alpha slices to validate
};

cudaError_t launch_init(int model, const InitArgs &a, int num_sms, cudaStream_t st);
cudaError_t launch_validate_alpha(const InitArgs &a, int num_sms, cudaStream_t st);
cudaError_t launch_wait_selftest(int *d_err, cudaStream_t st);

// Message returned by asets_last_error() on the calling thread.
void set_last_error(const char *msg);

// ---------------------------------------------------------------- context
EncodeTiledFn context_encoder(asets_context *ctx);
int context_num_sms(asets_context *ctx);
int context_device(asets_context *ctx);
cudaStream_t context_stream(asets_context *ctx);
// Memory pool of the context's short-lived scratch (nullptr if it cannot be made).
cudaMemPool_t context_pool(asets_context *ctx);

// ---------------------------------------------------------------- warm-start net
// One 3x3x3 convolution, 16 -> 16 channels (conv_tc.cu).
// Multilevel solve: grid geometry of one level (padded layout) and a
// fine/coarse pair.
constexpr int kMaxLevels = 8;
constexpr int kMinCoarseCells = 4;
struct GridGeom {
    int nr, nc, ns;
    long long pitch, plane, cells;
};
struct GridXfer {
    GridGeom f, c;
};
cudaError_t launch_restrict(const GridXfer &X, const float *src, float *dst, int labels,
                            float scale, int num_sms, cudaStream_t st);
cudaError_t launch_prolong(const GridXfer &X, const float *src, float *dst, int labels,
                           float scale, int axis, int num_sms, cudaStream_t st);

struct ConvLaunch {
    const void *x;       // BF16 [z][x][y][16]
    const void *w;       // BF16 [27][16 in][16 out], tap = (dz*3 + dx)*3 + dy
    const float *bias;   // [16] or null
    const void *mask;    // BF16 [v][16] or null: output *= (mask > 0)
    const float *addend = nullptr;  // FP32 [v][16] or null: added before ReLU/mask
    void *y;             // BF16 or FP32 [v][16]
    int ny, nx, nz;
    int relu, out_fp32, flip;
    // BF16 activation layouts: 0 channels-last [z][x][y][16]; 1 half-planar
    // [z][x][channel half][y][8] (each (z, x) row of a channel half one
    // contiguous run, so the convolution's row loads are long bursts).  `x`
    // and `mask` follow hp_in, a BF16 `y` hp_out; FP32 arrays are always
    // channels-last.
    int hp_in = 0, hp_out = 0;
};
cudaError_t launch_conv3_tc(EncodeTiledFn encode, const ConvLaunch &c, int num_sms,
                            cudaStream_t st, int *d_err);
int conv_smem_bytes();

}  // namespace asets
