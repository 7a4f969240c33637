// Internal interfaces between the host runtime and the kernel translation
// units of libasetscuda.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "kernel_args.h"

namespace asets {

// ---------------------------------------------------------------- stencil
// One compiled instance of stencil_iteration_kernel.
struct StencilVariant {
    int dim, epi, exact;
    int tr, tc, nt, nstage;
    int smem_bytes;   // dynamic shared memory per block
    int box_rows;     // TMA box rows (tr + 8)
    int box_cols;     // TMA box columns for slots other than SL_BC
    int box_cols_bc;  // TMA box columns of the SL_BC slot
    const void *fn;
};

// Variant tables, one per translation unit.
const StencilVariant *binary3d_variants(int *count);
const StencilVariant *binary2d_variants(int *count);
const StencilVariant *flow3d_variants(int *count);
const StencilVariant *flow2d_variants(int *count);

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
    int pitch, nr, nlab;
    float cc, inv_cc, inv_cc_l;  // 1/cc and 1/(cc*L) as the reference rounds them
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

// Message returned by asets_last_error() on the calling thread.
void set_last_error(const char *msg);

}  // namespace asets
