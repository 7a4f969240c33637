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

// The reference's norm rounded to float, fpt = (float)sqrt(0.5 * s) with s
// the double sum of the N squared face flows in order, computed in float.
// The exact sum of squares is formed as an unevaluated pair hi + lo (each
// square split exactly by FMA, the sums by TwoSum -- Knuth's error-free
// addition -- with the error terms added into lo; |hi + lo - S| <= 2^-40 S
// for N <= 6), renormalised so that |lo| <= ulp(hi)/2.  Then
// y0 = RN(sqrt(hi/2)) lies within one ulp of sqrt(S/2), its residual
// hi/2 - y0^2 is exact under FMA, and d ~ sqrt(S/2) - y0 to within 2^-17 of
// an ulp of y0, which picks y0 or a neighbour.  The double computation lies
// within 4 * 2^-53 (relative) of sqrt(S/2), so both round to the same float
// unless sqrt(S/2) is within 2^-12 of half a spacing of a rounding midpoint
// (below a power of two the spacing halves); then, and for sums outside
// [2^-60, 2^120], it returns false and the caller takes the double path.
// About 2^-12 of the evaluations near capacity do.
template <int N>
__device__ __forceinline__ bool ref_norm_f32(const float (&f)[N], float &out)
{
    float hi = __fmul_rn(f[0], f[0]);
    float lo = __fmaf_rn(f[0], f[0], -hi);
#pragma unroll
    for (int i = 1; i < N; ++i) {
        const float ph = __fmul_rn(f[i], f[i]);
        const float pl = __fmaf_rn(f[i], f[i], -ph);
        const float sum = __fadd_rn(hi, ph);
        const float bv = __fsub_rn(sum, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(sum, bv)), __fsub_rn(ph, bv));
        hi = sum;
        lo = __fadd_rn(lo, __fadd_rn(pl, err));
    }
    if (!(hi >= 0x1p-60f && hi <= 0x1p120f))
        return false;
    {
        // renormalise (Fast2Sum, exact as |hi| >= |lo|)
        const float s2 = __fadd_rn(hi, lo);
        lo = __fsub_rn(lo, __fsub_rn(s2, hi));
        hi = s2;
    }
    const float h2 = __fmul_rn(hi, 0.5f);
    const float y0 = __fsqrt_rn(h2);
    const float r = __fadd_rn(__fmaf_rn(-y0, y0, h2), __fmul_rn(lo, 0.5f));
    const float d = __fmul_rn(__fmul_rn(r, 0.5f), __frcp_rn(y0));
    const int yb = __float_as_int(y0);
    const float up = __int_as_float(yb + 1);
    // half the spacing to the neighbour on d's side
    float hs = __fmul_rn(__fsub_rn(up, y0), 0.5f);
    if (d < 0.0f && (yb & 0x7fffff) == 0)
        hs = __fmul_rn(hs, 0.5f);
    const float ad = fabsf(d);
    if (fabsf(__fsub_rn(ad, hs)) <= __fmul_rn(hs, 0x1p-12f))
        return false;  // too close to a midpoint to decide in float
    out = (ad < hs) ? y0 : __int_as_float(d > 0.0f ? yb + 1 : yb - 1);
    return true;
}

// The reference's fpt from its own double computation (the undecided
// cases of ref_norm_f32).  Not inlined, so that the compiler cannot hoist its
// conversions and double additions out of the rare branch that needs them.
template <int N>
__device__ __noinline__ float ref_norm_f64(const float *f)
{
    double s = (double)f[0] * (double)f[0];
    for (int i = 1; i < N; ++i)
        s = s + (double)f[i] * (double)f[i];
    return (float)__dsqrt_rn(s * 0.5);
}

template <>
struct Proj<true> {
    // Most voxels are far inside the constraint |p| <= alpha, where the
    // reference's factor is exactly 1 (fpt <= alpha).  A float sum of the
    // squares (relative error below 7 * 2^-24) decides that case: if
    // 0.5 * s * (1 + 2^-16) < alpha^2 in float, the double |p| of the
    // reference is below alpha as well (the margin exceeds both sums'
    // rounding), so its float fpt is <= alpha and the factor is 1.  The
    // other voxels -- the flow at or near its capacity -- get the
    // reference's float fpt from ref_norm_f32, or in the rare undecidable
    // cases from the reference's own double computation: the same bits as
    // the reference, mostly at FP32 cost.
    __device__ __forceinline__ static bool surely_inside(float s, float alpha)
    {
        const float lhs = __fmul_rn(__fmul_rn(s, 0.5f), 1.0f + 0x1p-16f);
        return lhs < __fmul_rn(alpha, alpha);
    }
    template <int N>
    __device__ __forceinline__ static float factor(const float (&f)[N], float alpha)
    {
        float sf = __fmul_rn(f[0], f[0]);
#pragma unroll
        for (int i = 1; i < N; ++i)
            sf = __fmaf_rn(f[i], f[i], sf);
        // All faces zero: fpt = 0 is not above alpha >= 0, so the factor is 1.
        // This is also every cell outside the volume (zero flows and zero
        // alpha from the tile loads' out-of-range fill).
        if (sf == 0.0f && alpha >= 0.0f)
            return 1.0f;
        if (surely_inside(sf, alpha))
            return 1.0f;
        float fpt;
        if (!ref_norm_f32<N>(f, fpt))
            fpt = ref_norm_f64<N>(f);
        return finish(fpt, alpha);
    }
    // faces in the reference's summation order
    __device__ __forceinline__ static float gk(float f0, float f1, float f2, float f3, float alpha)
    {
        const float f[4] = {f0, f1, f2, f3};
        return factor<4>(f, alpha);
    }
    __device__ __forceinline__ static float gk(float f0, float f1, float f2, float f3, float f4,
                                               float f5, float alpha)
    {
        const float f[6] = {f0, f1, f2, f3, f4, f5};
        return factor<6>(f, alpha);
    }
    // fpt -> 1 / (fpt / alpha) when fpt > alpha, else 1, in float as the
    // reference (maxflow/asetsBinaryMF3D_mex.c:317-331)
    __device__ __forceinline__ static float finish(float fpt, float alpha)
    {
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
