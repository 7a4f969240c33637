// End of an ALM iteration: block partials of erriter are summed in a fixed
// order by the last block to finish, which records cvg[it], applies the
// reference's stopping rule and advances the iteration counter.
#pragma once

#include "device_common.cuh"
#include "kernel_args.h"

namespace asets {

// done_count (or null): counter of finished problems of a batch, bumped when
// this problem finishes.
template <int NT>
__device__ __forceinline__ void finish_iteration(float erru, IterControl *ctl, double *partials,
                                                 float *cvg, int it, double *s_red,
                                                 int *s_is_last, unsigned int *done_count)
{
    const double part = block_sum_double<NT>(erru, s_red);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = part;
        __threadfence();
        const unsigned int ticket = atomicAdd(&ctl->ticket, 1u);
        *s_is_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (*s_is_last && threadIdx.x < 32) {
        __threadfence();
        double acc = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += 32)
            acc += __ldcg(partials + b);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) {
            // cvg[i] = total_err / (float)N with total_err a float
            // (maxflow/asetsBinaryMF3D_mex.c:183)
            const float c = __fdiv_rn((float)acc, ctl->denom);
            cvg[it] = c;
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
                if (done_count)
                    atomicAdd(done_count, 1u);
            }
            __threadfence();
        }
    }
}

}  // namespace asets
