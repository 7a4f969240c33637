// Test helper: the tensor-core weight and bias gradients of a 3x3x3, 16 -> 16
// convolution (asets::launch_wgrad_tc) against a double-precision reference
// on the GPU, on seeded BF16 activations and output gradients.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "wgrad_tc.cuh"

// element index of (z, x, y, channel c): channels-last, or half-planar with
// rows padded to ypad
__device__ __forceinline__ long long at(int hp, int ny, int nx, int z, int x, int y, int c)
{
    const long long zx = (long long)z * nx + x;
    if (!hp)
        return (zx * ny + y) * 16 + c;
    const long long yp = (ny + 7) / 8 * 8;
    return (zx * 2 + c / 8) * yp * 8 + (long long)y * 8 + (c & 7);
}

// reference: one thread per (tap, ci, co) or bias co, summing over all voxels in double
__global__ void wgrad_ref_kernel(const __nv_bfloat16 *a, const __nv_bfloat16 *g, int ny, int nx,
                                 int nz, int hp, double *dw, double *dabs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 27 * 256 + 16)
        return;
    const bool bias = i >= 27 * 256;
    const int t = i / 256, ci = (i / 16) % 16, co = bias ? i - 27 * 256 : i % 16;
    const int dz = t / 9 - 1, dx = (t / 3) % 3 - 1, dy = t % 3 - 1;
    double s = 0.0, sa = 0.0;
    for (int z = 0; z < nz; ++z)
        for (int x = 0; x < nx; ++x)
            for (int y = 0; y < ny; ++y) {
                const double gv = __bfloat162float(g[at(hp, ny, nx, z, x, y, co)]);
                double av = 1.0;
                if (!bias) {
                    const int zz = z + dz, xx = x + dx, yy = y + dy;
                    av = (zz >= 0 && zz < nz && xx >= 0 && xx < nx && yy >= 0 && yy < ny)
                             ? (double)__bfloat162float(a[at(hp, ny, nx, zz, xx, yy, ci)])
                             : 0.0;
                }
                s += av * gv;
                sa += fabs(av * gv);
            }
    dw[i] = s;
    dabs[i] = sa;
}

__global__ void fill_kernel(__nv_bfloat16 *p, long long n, unsigned long long seed)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        unsigned long long z = seed + (unsigned long long)i * 0x9e3779b97f4a7c15ull;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        p[i] = __float2bfloat16_rn((float)((int)(z >> 40) - (1 << 23)) * 0x1p-23f);
    }
}

// the padding voxels of a half-planar array are zero
__global__ void zero_pad_kernel(__nv_bfloat16 *p, int ny, int nx, int nz)
{
    const long long yp = (ny + 7) / 8 * 8;
    const long long n = yp * nx * nz * 16;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        if ((i / 8) % yp >= ny)
            p[i] = __float2bfloat16_rn(0.f);
}

// Returns 0 and the largest |got - ref| / (sum |a*g| + 1e-30) over all
// outputs; hp: both operands half-planar with padded rows.
extern "C" __attribute__((visibility("default"))) int wgrad_check(int ny, int nx, int nz, int hp,
                                                                  double *worst_out)
{
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess || !fn)
        return 1;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long vox = (long long)((ny + 7) / 8 * 8) * nx * nz;  // with padding
    __nv_bfloat16 *a = nullptr, *g = nullptr;
    float *dw = nullptr, *partial = nullptr;
    double *ref = nullptr, *rabs = nullptr;
    int *err = nullptr;
    if (cudaMalloc(&a, vox * 32) || cudaMalloc(&g, vox * 32) ||
        cudaMalloc(&dw, (27 * 256 + 16) * 4) || cudaMalloc(&partial, (size_t)sms * 28 * 256 * 4) ||
        cudaMalloc(&ref, (27 * 256 + 16) * 8) || cudaMalloc(&rabs, (27 * 256 + 16) * 8) ||
        cudaMalloc(&err, 4))
        return 2;
    fill_kernel<<<256, 256>>>(a, vox * 16, 11);
    fill_kernel<<<256, 256>>>(g, vox * 16, 29);
    if (hp) {
        zero_pad_kernel<<<256, 256>>>(a, ny, nx, nz);
        zero_pad_kernel<<<256, 256>>>(g, ny, nx, nz);
    }
    cudaMemset(dw, 0, (27 * 256 + 16) * 4);
    cudaMemset(err, 0, 4);
    if (asets::launch_wgrad_tc(reinterpret_cast<asets::EncodeTiledFn>(fn), a, g, dw, dw + 27 * 256,
                               ny, nx, nz, partial, sms, err, 0, hp) != cudaSuccess)
        return 3;
    wgrad_ref_kernel<<<(27 * 256 + 16 + 127) / 128, 128>>>(a, g, ny, nx, nz, hp, ref, rabs);
    if (cudaDeviceSynchronize() != cudaSuccess)
        return 4;
    int herr = 0;
    cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost);
    if (herr)
        return 5;
    std::vector<float> got(27 * 256 + 16);
    std::vector<double> r(27 * 256 + 16), ra(27 * 256 + 16);
    cudaMemcpy(got.data(), dw, got.size() * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(r.data(), ref, r.size() * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(ra.data(), rabs, ra.size() * 8, cudaMemcpyDeviceToHost);
    double worst = 0.0;
    for (size_t i = 0; i < got.size(); ++i) {
        const double e = fabs((double)got[i] - r[i]) / (ra[i] + 1e-30);
        if (e > worst)
            worst = e;
    }
    *worst_out = worst;
    cudaFree(a);
    cudaFree(g);
    cudaFree(dw);
    cudaFree(partial);
    cudaFree(ref);
    cudaFree(rabs);
    cudaFree(err);
    return 0;
}
