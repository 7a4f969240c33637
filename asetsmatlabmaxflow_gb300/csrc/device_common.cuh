// Device-side building blocks shared by the solver kernels: TMA tiled loads,
// mbarriers with bounded waits, and the reference's float arithmetic.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernel_args.h"

namespace asets {

// Budget of every spin-wait in these kernels: a tile load takes
// microseconds, so one second means the copy is lost.
constexpr unsigned long long kWaitBudgetNs = 1000000000ull;

__device__ __forceinline__ unsigned long long global_timer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------- mbarrier
__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t phase)
{
    uint32_t ok;
    // the thread may sleep in try_wait for up to the hint (ns) before retrying
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase), "r"(20000u)
        : "memory");
    return ok != 0;
}

// Wait for `phase` of `bar` to complete, giving up after kWaitBudgetNs.
// Returns false on timeout.  `abort_flag` (shared) short-cuts the wait once
// another thread of the block has already given up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t phase,
                                                  volatile int *abort_flag)
{
    if (mbar_try_wait(bar, phase))
        return true;
    const unsigned long long t0 = global_timer_ns();
    while (true) {
        if (mbar_try_wait(bar, phase))
            return true;
        if (*abort_flag)
            return false;
        if (global_timer_ns() - t0 > kWaitBudgetNs) {
            *abort_flag = 1;
            return false;
        }
    }
}

// ---------------------------------------------------------------- TMA
// 4D tiled load of one box into shared memory, completing on `bar`.
// Coordinates: {row, col, plane, label}; out-of-range elements read as 0.
// The row coordinate must be a multiple of 4 (16 bytes of fp32).
__device__ __forceinline__ void tma_load_4d(void *smem_dst, const CUtensorMap *map, int c0, int c1,
                                            int c2, int c3, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_addr(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
        "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap *map)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// ---------------------------------------------------------------- arithmetic
// The kernels are compiled with --fmad=false, so `a*b + c` is a rounded
// multiply followed by a rounded add, as in the reference's SSE code.

// |p(x)| -> gk of projStep (maxflow/asetsBinaryMF3D_mex.c:317-331) for the
// face sum s2 = sum of squared face flows.  EXACT forms the sum and the root
// in double with the reference's order; the fast path uses float.
template <bool EXACT>
struct Proj;

template <>
struct Proj<true> {
    // faces in the reference's summation order
    __device__ __forceinline__ static float gk(float f0, float f1, float f2, float f3, float alpha)
    {
        double s = (double)f0 * (double)f0;
        s = s + (double)f1 * (double)f1;
        s = s + (double)f2 * (double)f2;
        s = s + (double)f3 * (double)f3;
        return finish(s, alpha);
    }
    __device__ __forceinline__ static float gk(float f0, float f1, float f2, float f3, float f4,
                                               float f5, float alpha)
    {
        double s = (double)f0 * (double)f0;
        s = s + (double)f1 * (double)f1;
        s = s + (double)f2 * (double)f2;
        s = s + (double)f3 * (double)f3;
        s = s + (double)f4 * (double)f4;
        s = s + (double)f5 * (double)f5;
        return finish(s, alpha);
    }
    __device__ __forceinline__ static float finish(double s, float alpha)
    {
        float fpt = (float)__dsqrt_rn(s * 0.5);
        fpt = (fpt > alpha) ? __fdiv_rn(fpt, alpha) : 1.0f;
        return __fdiv_rn(1.0f, fpt);
    }
};

template <>
struct Proj<false> {
    __device__ __forceinline__ static float gk(float f0, float f1, float f2, float f3, float alpha)
    {
        float s = __fmul_rn(f0, f0);
        s = __fmaf_rn(f1, f1, s);
        s = __fmaf_rn(f2, f2, s);
        s = __fmaf_rn(f3, f3, s);
        return finish(s, alpha);
    }
    __device__ __forceinline__ static float gk(float f0, float f1, float f2, float f3, float f4,
                                               float f5, float alpha)
    {
        float s = __fmul_rn(f0, f0);
        s = __fmaf_rn(f1, f1, s);
        s = __fmaf_rn(f2, f2, s);
        s = __fmaf_rn(f3, f3, s);
        s = __fmaf_rn(f4, f4, s);
        s = __fmaf_rn(f5, f5, s);
        return finish(s, alpha);
    }
    __device__ __forceinline__ static float finish(float s, float alpha)
    {
        // min(1, alpha/|p|) from the hardware reciprocal square root: equal
        // to the reference's (|p| > alpha ? 1/(|p|/alpha) : 1) up to a few
        // roundings (|p| = 0 gives alpha*inf = inf, so 1).
        return fminf(1.0f, alpha * rsqrtf(s * 0.5f));
    }
};

// x / d rounded to nearest for a fixed divisor, given rd = RN(1/d).
// Markstein's correction (Markstein, "Computation of elementary functions on
// the IBM RISC System/6000", 1990): with q = RN(x*rd) within one ulp of x/d,
// the residual x - q*d is exact under FMA and q + residual*rd rounds to
// RN(x/d).  It needs every intermediate in the normal range, so x outside
// [2^-100, 2^100] in magnitude (zero, tiny, huge, non-finite) takes the IEEE
// division.  tests/test_gpu_kernels.py compares it with __fdiv_rn over all
// 2^32 inputs for several divisors.
__device__ __forceinline__ float div_by(float x, float d, float rd)
{
    const float ax = fabsf(x);
    if (ax == 0.0f)
        return __fmul_rn(x, rd);  // +-0: the IEEE quotient keeps the sign
    if (ax >= 0x1p-100f && ax <= 0x1p100f) {
        const float q = __fmul_rn(x, rd);
        const float r = __fmaf_rn(-q, d, x);
        return __fmaf_rn(r, rd, q);
    }
    return __fdiv_rn(x, d);
}

// u/cc: EXACT takes the correctly rounded quotient (the reference's float
// division); the fast path multiplies by the rounded reciprocal (within one
// ulp of it).
template <bool EXACT>
__device__ __forceinline__ float div_cc(float x, float cc, float inv_cc)
{
    if constexpr (EXACT)
        return div_by(x, cc, inv_cc);
    else
        return x * inv_cc;
}

// MIN of the reference macros: `a < b ? a : b` (NaN picks b).
__device__ __forceinline__ float min_ref(float a, float b) { return (a < b) ? a : b; }
// ABS of the reference macros; identical to fabsf except for the sign of a NaN.
__device__ __forceinline__ float abs_ref(float x) { return fabsf(x); }

// EXACT keeps the reference's select and MIN forms; the fast path zeroes a
// border term by multiplying with a 0/1 mask (FMA pipe instead of the
// half-rate ALU pipe) and takes the hardware min.
template <bool EXACT>
__device__ __forceinline__ float keep_if(float v, bool ok, float okf)
{
    if constexpr (EXACT)
        return ok ? v : 0.0f;
    else
        return v * okf;
}
template <bool EXACT>
__device__ __forceinline__ float min_sel(float a, float b)
{
    if constexpr (EXACT)
        return min_ref(a, b);
    else
        return fminf(a, b);
}

// Warp + block sum of a per-thread float into one double (lane order fixed).
template <int NT>
__device__ __forceinline__ double block_sum_double(float v, double *scratch)
{
    double d = (double)v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        d += __shfl_xor_sync(0xffffffffu, d, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        scratch[warp] = d;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0) {
        for (int w = 0; w < NT / 32; ++w)
            t += scratch[w];
    }
    return t;  // valid in thread 0
}

}  // namespace asets
