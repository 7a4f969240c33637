// Weight and bias gradients of a 3x3x3, 16 -> 16 channel convolution on the
// 5th-generation tensor cores (tcgen05), BF16 operands, FP32 accumulation.
//
//   dW[t][ci][co] = sum_v a[v + off_t][ci] * g[v][co],   db[co] = sum_v g[v][co]
//
// is, per tap t, a GEMM with the voxels as the reduction axis K:
// D_t[co][ci] = sum_v G[co][v] * A_t[v][ci].  Both operands are read in the
// layout the forward kernel stages (conv_tc.cu): [channel half][voxel][8
// channels], i.e. 8 channels contiguous per voxel -- MN-major operands
// (instruction descriptor bits 15 and 16).  A tap's shift is then an offset
// along the voxels, never along the 16-byte inner dimension the TMA loads
// are aligned on.  A is the output gradient tile (M = co), B the activation
// rows of the tap (N = ci = 16, K = 16 voxels per MMA).  M must be 64 or 128
// for one CTA; the MMAs run with M = 128 and only D rows 0..15 (co) are
// used -- rows 16..127 multiply whatever follows the gradient tile in shared
// memory (always inside the allocation) and are discarded.  A 28th "tap"
// multiplies G by a constant block of ones: its column 0 is the bias
// gradient.  28 accumulators of 16 FP32 columns = 448 TMEM columns.
//
// Persistent grid, one CTA per SM (the shared memory use keeps it so);
// a CTA walks 128-voxel rows along y, three TMA stages deep; one thread
// issues 224 MMAs per row and the refill of the previous row's stage once
// that row's MMAs have committed.  At the end each CTA writes its 28 x 16 x
// 16 partial sums, and a second kernel adds the CTAs' partials in a fixed
// order into dW and db (deterministic).
#pragma once

#include <cuda_bf16.h>

#include <cstring>

#include "internal.h"
#include "tcgen05.cuh"

namespace asets {

constexpr int kWgtThreads = 128;
constexpr int kWgtStages = 3;
constexpr int kWgtTaps = 28;                               // 27 taps + bias
// staged activation rows: 130 voxels y-1 .. y+128 (channels-last input) or
// 144 voxels y-8 .. y+135 (half-planar input, 128-byte loads), as in conv_tc.cu
constexpr int kWgtActStride = (9 * 2 * 144 * 16 + 127) / 128 * 128;  // 41,472
constexpr int kWgtGradBytes = 2 * 128 * 16;                // [half][128 voxels][8 co]
constexpr int kWgtOnesBytes = 512;                         // [2 halves][16 voxels][8] ones
// gradient stages first: an M = 128 A operand reads 16 core-matrix rows
// 2,048 B apart from a stage's base, 32 KB, which the later regions cover
constexpr int kWgtGradOff = 0;
constexpr int kWgtOnesOff = kWgtStages * kWgtGradBytes;
constexpr int kWgtActOff = kWgtOnesOff + kWgtOnesBytes;
constexpr int kWgtSmem = kWgtActOff + kWgtStages * kWgtActStride + 128;
static_assert(kWgtGradOff + (kWgtStages - 1) * kWgtGradBytes + 16 * 2048 <= kWgtSmem - 128,
              "the padded A operand must stay inside the shared memory");

struct WgradTcArgs {
    CUtensorMap act;     // the BF16 input, staged 3x3 rows as [row][half][voxel][8]
    CUtensorMap grad;    // the BF16 output gradient, staged [half][128 voxels][8]
    float *partial;      // [gridDim.x][28][16 ci][16 co]
    int *err;
    int ny, nx, nz, ytiles;
    int hp;                                  // half-planar operands
    int act_half, act_row, act_bytes, vox_base;
};

__global__ void __launch_bounds__(kWgtThreads, 1)
    wgrad_tc_kernel(const __grid_constant__ WgradTcArgs A)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t full_bar[kWgtStages], mma_bar[kWgtStages];
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        s_abort = 0;
        for (int i = 0; i < kWgtStages; ++i) {
            mbar_init(&full_bar[i], 1);
            mbar_init(&mma_bar[i], 1);
        }
        mbar_fence_init();
    }
    // the block of ones (bias gradient), BF16 1.0
    for (int i = tid; i < kWgtOnesBytes / 2; i += kWgtThreads)
        reinterpret_cast<unsigned short *>(smem + kWgtOnesOff)[i] = 0x3F80u;
    if (warp == 0)
        tmem_alloc(&s_tmem, 512);
    fence_proxy_async_smem();
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    const uint32_t tmem = s_tmem;

    const int ntiles = A.ytiles * A.nx * A.nz;
    // tiles of this CTA: blockIdx.x, blockIdx.x + gridDim.x, ...
    const int mine = ((int)blockIdx.x < ntiles) ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    // M = 128, N = 16, both operands MN-major
    const uint32_t idesc = umma_idesc_bf16_f32(128, 16) | (1u << 15) | (1u << 16);
    auto issue = [&](int j) {
        const int tile = blockIdx.x + j * gridDim.x;
        const int st = j % kWgtStages;
        const int yt = tile % A.ytiles, rest = tile / A.ytiles;
        const int x = rest % A.nx, z = rest / A.nx;
        mbar_arrive_expect_tx(&full_bar[st], A.act_bytes + kWgtGradBytes);
        tma_load_5d(smem + kWgtActOff + st * kWgtActStride, &A.act, 0,
                    A.hp ? yt * 16 - 1 : yt * 128 - 1, 0, x - 1, z - 1, &full_bar[st]);
        tma_load_5d(smem + kWgtGradOff + st * kWgtGradBytes, &A.grad, 0, A.hp ? yt * 16 : yt * 128,
                    0, x, z, &full_bar[st]);
    };

    bool ok = true;
    int issued = 0;
    if (tid == 0) {
        for (; issued < kWgtStages && issued < mine; ++issued)
            issue(issued);
        const uint32_t ones = smem_addr(smem + kWgtOnesOff);
        for (int j = 0; j < mine && ok; ++j) {
            const int st = j % kWgtStages;
            const uint32_t ph = (j / kWgtStages) & 1;
            ok = mbar_wait_bounded(&full_bar[st], ph, &s_abort);
            if (!ok)
                break;
            tc_fence_after_sync();
            const uint32_t g0 = smem_addr(smem + kWgtGradOff + st * kWgtGradBytes);
            const uint32_t a0 =
                smem_addr(smem + kWgtActOff + st * kWgtActStride) + (A.vox_base - 1) * 16;
            for (int ks = 0; ks < 8; ++ks) {  // 16 voxels per MMA
                // A: co x voxels, core matrices 8 voxels x 8 co; K step 128 B, M step 2,048 B
                const uint64_t ad = umma_smem_desc(g0 + ks * 256, 128, 2048);
                const uint32_t acc = (j > 0 || ks > 0) ? 1u : 0u;
                for (int t = 0; t < 27; ++t) {
                    const int dz = t / 9, dx = (t / 3) % 3, dy = t % 3;
                    // B: ci x voxels of the tap's row, shifted by dy; N step: channel half
                    const uint32_t b = a0 + (dz * 3 + dx) * A.act_row + (dy + 16 * ks) * 16;
                    const uint64_t bd = umma_smem_desc(b, 128, A.act_half);
                    umma_bf16(tmem + t * 16, ad, bd, idesc, acc);
                }
                umma_bf16(tmem + 27 * 16, ad, umma_smem_desc(ones, 128, 256), idesc, acc);
            }
            umma_commit(&mma_bar[st]);
            // refill the previous row's stage once its MMAs are done
            if (j >= 1 && issued < mine) {
                const int sp = (j - 1) % kWgtStages;
                ok = mbar_wait_bounded(&mma_bar[sp], ((j - 1) / kWgtStages) & 1, &s_abort);
                if (ok)
                    issue(issued++);
            }
        }
        // the last row's MMAs (and with them all earlier ones) have finished
        if (ok && mine > 0)
            ok = mbar_wait_bounded(&mma_bar[(mine - 1) % kWgtStages], ((mine - 1) / kWgtStages) & 1,
                                   &s_abort);
        if (!ok) {
            atomicOr(A.err, 1);
            // drain the copies still in flight (bounded)
            s_abort = 0;
            for (int j = 0; j < issued; ++j)
                mbar_wait_bounded(&full_bar[j % kWgtStages], (j / kWgtStages) & 1, &s_abort);
        }
    }
    tc_fence_before_sync();
    const bool good = !__syncthreads_or(!ok);
    tc_fence_after_sync();
    if (good && warp == 0) {
        // rows 0..15 of each accumulator (lanes 0..15): D_t[co][ci]
        float *P = A.partial + (size_t)blockIdx.x * kWgtTaps * 256;
        for (int t = 0; t < kWgtTaps; ++t) {
            float v[16];
            tmem_load16(tmem + t * 16, v);
            if (lane < 16) {
                if (mine == 0) {
#pragma unroll
                    for (int ci = 0; ci < 16; ++ci)
                        v[ci] = 0.f;
                }
#pragma unroll
                for (int ci = 0; ci < 16; ++ci)
                    P[(t * 16 + ci) * 16 + lane] = v[ci];
            }
        }
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    if (warp == 0)
        tmem_dealloc(tmem, 512);
}

// dW[t][ci][co] += sum over CTAs of the partials (tap 27, ci 0: the bias).
__global__ void wgrad_tc_reduce_kernel(const float *partial, int nblocks, float *dw, float *db)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 27 * 256 + 16)
        return;
    const int src = (i < 27 * 256) ? i : 27 * 256 + (i - 27 * 256);  // bias: ci 0 of tap 27
    float s = 0.f;
    for (int b = 0; b < nblocks; ++b)
        s += partial[(size_t)b * kWgtTaps * 256 + src];
    if (i < 27 * 256)
        dw[i] += s;
    else
        db[i - 27 * 256] += s;
}

// Tensor maps of the two operands, the launch, the reduction.  `partial`
// holds num_sms x 28 x 256 floats.  `hp`: both BF16 arrays half-planar
// ([z][x][half][y][8]) instead of channels-last ([z][x][y][16]).
inline cudaError_t launch_wgrad_tc(EncodeTiledFn encode, const __nv_bfloat16 *act,
                                   const __nv_bfloat16 *grad, float *dw, float *db, int ny, int nx,
                                   int nz, float *partial, int num_sms, int *d_err,
                                   cudaStream_t st, int hp = 0)
{
    WgradTcArgs A;
    memset(&A, 0, sizeof A);
    const int ypad = (ny + 7) / 8 * 8;
    // channels-last: (8 ch, y, half, x, z); half-planar [z][x][half][ypad][8]:
    // (8 voxels x 8 ch, ypad / 8, half, x, z)
    cuuint64_t dims[5] = {8, (cuuint64_t)ny, 2, (cuuint64_t)nx, (cuuint64_t)nz};
    cuuint64_t strides[4] = {32, 16, (cuuint64_t)32 * ny, (cuuint64_t)32 * ny * nx};
    cuuint32_t box_a[5] = {8, 130, 2, 3, 3};
    cuuint32_t box_g[5] = {8, 128, 2, 1, 1};
    if (hp) {
        const cuuint64_t d[5] = {64, (cuuint64_t)ypad / 8, 2, (cuuint64_t)nx, (cuuint64_t)nz};
        const cuuint64_t s[4] = {128, (cuuint64_t)16 * ypad, (cuuint64_t)32 * ypad,
                                 (cuuint64_t)32 * ypad * nx};
        const cuuint32_t ba[5] = {64, 18, 2, 3, 3}, bg[5] = {64, 16, 2, 1, 1};
        memcpy(dims, d, sizeof d);
        memcpy(strides, s, sizeof s);
        memcpy(box_a, ba, sizeof ba);
        memcpy(box_g, bg, sizeof bg);
    }
    cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    CUresult r = encode(&A.act, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<__nv_bfloat16 *>(act),
                        dims, strides, box_a, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    r = encode(&A.grad, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<__nv_bfloat16 *>(grad), dims,
               strides, box_g, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    A.partial = partial;
    A.err = d_err;
    A.ny = ny;
    A.nx = nx;
    A.nz = nz;
    A.ytiles = (ny + 127) / 128;
    A.hp = hp;
    const int vox = hp ? 144 : 130;
    A.act_half = vox * 16;
    A.act_row = 2 * vox * 16;
    A.act_bytes = 9 * A.act_row;
    A.vox_base = hp ? 8 : 1;
    cudaError_t e = cudaFuncSetAttribute(wgrad_tc_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, kWgtSmem);
    if (e != cudaSuccess)
        return e;
    const int tiles = A.ytiles * nx * nz;
    const int grid = tiles < num_sms ? tiles : num_sms;
    wgrad_tc_kernel<<<grid, kWgtThreads, kWgtSmem, st>>>(A);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    wgrad_tc_reduce_kernel<<<(27 * 256 + 16 + 255) / 256, 256, 0, st>>>(partial, grid, dw, db);
    return cudaGetLastError();
}

}  // namespace asets
