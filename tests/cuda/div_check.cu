// Test helper: compares asets::div_by (Markstein-corrected reciprocal
// division used by the iteration kernels) with IEEE __fdiv_rn over every
// 32-bit pattern of the dividend, for one divisor.
#include <cstdint>

#include "device_common.cuh"

__global__ void div_check_kernel(float d, float rd, unsigned long long *mismatch,
                                 unsigned int *first_bad)
{
    unsigned long long local = 0;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < (1ull << 32); i += stride) {
        const float x = __uint_as_float((unsigned int)i);
        const float a = asets::div_by(x, d, rd);
        const float b = __fdiv_rn(x, d);
        const bool same = (__float_as_uint(a) == __float_as_uint(b)) || (a != a && b != b);
        if (!same) {
            ++local;
            atomicMin(first_bad, (unsigned int)i);
        }
    }
    if (local)
        atomicAdd(mismatch, local);
}

extern "C" __attribute__((visibility("default"))) int div_check(float d, unsigned long long *mismatch_out, unsigned int *first_bad_out)
{
    unsigned long long *m = nullptr;
    unsigned int *f = nullptr;
    if (cudaMalloc(&m, sizeof *m) != cudaSuccess || cudaMalloc(&f, sizeof *f) != cudaSuccess)
        return 1;
    cudaMemset(m, 0, sizeof *m);
    cudaMemset(f, 0xff, sizeof *f);
    const float rd = 1.0f / d;
    div_check_kernel<<<152 * 8, 256>>>(d, rd, m, f);
    if (cudaDeviceSynchronize() != cudaSuccess)
        return 2;
    cudaMemcpy(mismatch_out, m, sizeof *m, cudaMemcpyDeviceToHost);
    cudaMemcpy(first_bad_out, f, sizeof *f, cudaMemcpyDeviceToHost);
    cudaFree(m);
    cudaFree(f);
    return 0;
}
