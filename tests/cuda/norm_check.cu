// Test helper: compares the projection factor of the EXACT kernels
// (asets::Proj<true>: a float pre-check, the reference's double norm
// reproduced in float by asets::ref_norm_f32, and the double computation
// for the undecided cases) with the reference's double computation itself
// (maxflow/asetsBinaryMF3D_mex.c:317-331), on seeded pseudo-random face
// flows and capacities.
#include <cstdint>

#include "device_common.cuh"

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    // SplitMix64 finaliser (Steele, Lea and Flood, "Fast splittable
    // pseudorandom number generators", 2014)
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ float unit(uint64_t h)  // [-1, 1)
{
    return (float)((int)(uint32_t)(h >> 40) - (1 << 23)) * 0x1p-23f;
}

template <int N>
__device__ float ref_factor(const float (&f)[N], float alpha)
{
    double s = (double)f[0] * (double)f[0];
#pragma unroll
    for (int i = 1; i < N; ++i)
        s = s + (double)f[i] * (double)f[i];
    float fpt = (float)__dsqrt_rn(s * 0.5);
    fpt = (fpt > alpha) ? __fdiv_rn(fpt, alpha) : 1.0f;
    return __fdiv_rn(1.0f, fpt);
}

template <int N>
__global__ void norm_check_kernel(uint64_t n, int mode, uint64_t seed,
                                  unsigned long long *mismatch)
{
    unsigned long long local = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t h = mix64(seed ^ (i * 0x9e3779b97f4a7c15ull));
        float f[N];
#pragma unroll
        for (int k = 0; k < N; ++k) {
            h = mix64(h + k + 1);
            float v = unit(h);
            if (mode == 1)
                v = ldexpf(v, (int)(h & 63) - 50);             // wide dynamic range
            else if (mode == 2 && k > 0)
                v = ldexpf(v, -12);                            // one dominant face
            else if (mode == 3)
                v = (float)((int)(v * 64.0f)) * 0.015625f;     // few-bit values (exact ties)
            f[k] = v;
        }
        h = mix64(h + 101);
        float alpha = 0.05f + 0.95f * fabsf(unit(h));
        if (mode == 4) {
            // norm within a few ulps of a power of two, capacity exactly that
            // power (flows at capacity where alpha is 1 or 0.5)
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < N; ++k)
                s += (double)f[k] * (double)f[k];
            alpha = (h & 2) ? 1.0f : 0.5f;
            const double target =
                (double)alpha * (1.0 + ldexp((double)((int)((h >> 8) & 31) - 16), -24));
            const double sc = (s > 0.0) ? target / sqrt(s * 0.5) : 1.0;
#pragma unroll
            for (int k = 0; k < N; ++k)
                f[k] = (float)((double)f[k] * sc);
        } else if (h & 1) {
            // a capacity within a few ulps of the norm: the comparison edge
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < N; ++k)
                s += (double)f[k] * (double)f[k];
            const float nf = (float)sqrt(s * 0.5);
            alpha = __int_as_float(__float_as_int(nf) + (int)((h >> 8) & 7) - 3);
            if (!(alpha > 0.0f))
                alpha = 1.0f;
        }
        float a;
        if constexpr (N == 4)
            a = asets::Proj<true>::gk(f[0], f[1], f[2], f[3], alpha);
        else
            a = asets::Proj<true>::gk(f[0], f[1], f[2], f[3], f[4], f[5], alpha);
        const float b = ref_factor<N>(f, alpha);
        if (__float_as_uint(a) != __float_as_uint(b) && !(a != a && b != b))
            ++local;
    }
    if (local)
        atomicAdd(mismatch, local);
}

extern "C" __attribute__((visibility("default"))) int norm_check(int nfaces, int mode,
                                                                 unsigned long long n,
                                                                 unsigned long long *mismatch_out)
{
    unsigned long long *m = nullptr;
    if (cudaMalloc(&m, sizeof *m) != cudaSuccess)
        return 1;
    cudaMemset(m, 0, sizeof *m);
    if (nfaces == 4)
        norm_check_kernel<4><<<152 * 8, 256>>>(n, mode, 0x5eed0000ull + mode, m);
    else
        norm_check_kernel<6><<<152 * 8, 256>>>(n, mode, 0x5eed1000ull + mode, m);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        cudaFree(m);
        return 2;
    }
    cudaMemcpy(mismatch_out, m, sizeof *m, cudaMemcpyDeviceToHost);
    cudaFree(m);
    return 0;
}
