// 3x3x3 convolutions of the learned warm start on the 5th-generation tensor
// cores (tcgen05): BF16 activations and weights, FP32 accumulation in TMEM.
//
// Activations are channels-last, 16 channels of BF16 per voxel
// ([z][x][y][16]).  A convolution is an implicit GEMM: an output tile is 128
// consecutive voxels along y at one (x, z) (M = 128), each of the 27 taps is
// one MMA with K = 16 input channels and N = 16 output channels, and the
// accumulator (128 x 16 FP32) lives in TMEM.  One 5D TMA load per tile stages
// the 3 x 3 neighbouring rows, y-1 .. y+128, zero-filled outside the volume
// (the convolution's zero padding), as [row][channel half][voxel][8 channels]:
// the no-swizzle K-major layout in which a tap's A operand is a plain offset.
//
// The same kernel computes the data gradient: with `flip` the taps are
// mirrored and the weight matrix transposed.  The weight gradient is a
// separate tcgen05 kernel (wgrad_tc.cuh).  The epilogue adds the bias and
// an optional FP32 addend (a second convolution's result), then applies ReLU
// and an optional mask (the ReLU derivative of the layer below).
#include <cuda_bf16.h>

#include <cstring>

#include "internal.h"
#include "tcgen05.cuh"

namespace asets {

constexpr int kConvThreads = 192;            // warp 0: TMA, warp 1: MMA, warps 2-5: epilogue
constexpr int kConvStages = 4;               // TMA ring depth
constexpr int kConvAcc = 8;                  // TMEM accumulators (16 FP32 columns each)
constexpr int kConvRows = 9;                 // (dz, dx) neighbour rows
// Staged voxels per row: channels-last input y-1 .. y+128 (130, loaded in
// 16-byte runs); half-planar input y-8 .. y+135 (144 = 18 groups of 8
// voxels, loaded in 128-byte runs from rows padded to a multiple of 8).
constexpr int kConvVoxCL = 130, kConvVoxHP = 144;
constexpr int kConvStageStride = (kConvRows * 2 * kConvVoxHP * 16 + 127) / 128 * 128;  // 41,472
constexpr int kConvTapBytes = 2 * 16 * 16;              // B operand of one tap
constexpr int kConvWBytes = 27 * kConvTapBytes;         // 13,824 B
// + 32 KB: operand descriptors can only address inside the allocation
constexpr int kConvSmem = kConvStages * kConvStageStride + kConvWBytes + 128 + 32768;

struct ConvTcArgs {
    CUtensorMap act;           // 5D view (8 ch, y, half, x, z) of the BF16 input
    const __nv_bfloat16 *w;    // [27][16 in][16 out]
    const float *bias;         // [16] or null
    const __nv_bfloat16 *mask; // [v][16] or null: output *= (mask > 0)
    const float *addend;       // [v][16] FP32 or null: added before ReLU and mask
    void *out;                 // [v][16] BF16 or FP32
    int *err;
    int ny, nx, nz, ytiles;
    int relu, out_fp32, flip;
    int hp_in, hp_out;         // half-planar BF16 input (and mask) / output
    int ypad;                  // half-planar row length (ny rounded up to 8)
    int half_bytes, row_bytes, stage_bytes;  // staged layout: [row][half][voxel][8]
    int vox_base;              // staged voxel of y - 1 is vox_base - 1 (1 or 8)
};

// Warp-specialised: warp 0 (one lane) keeps a ring of kConvStages tile
// stages loading, warp 1 (one lane) issues each tile's 27 MMAs into one of
// kConvAcc TMEM accumulators as soon as its stage and accumulator are free
// and commits them to the stage's "empty" and the accumulator's "full"
// barrier, and warps 2-5 (TMEM lane quarters 2, 3, 0, 1) drain full
// accumulators through the epilogue and hand them back.  No role waits on
// another's per-tile round trip, so the tensor core sees a steady stream
// of MMAs.  Every wait is bounded; a timeout raises the shared abort flag,
// every role leaves its loop, the producer waits (bounded) for its copies
// in flight and the MMA lane for its last commit before TMEM is freed.
__global__ void __launch_bounds__(kConvThreads, 1) conv3_tc_kernel(const __grid_constant__ ConvTcArgs A)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t full_bar[kConvStages], empty_bar[kConvStages];
    __shared__ uint64_t accf_bar[kConvAcc], acce_bar[kConvAcc];
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
    unsigned char *wsm = smem + kConvStages * kConvStageStride;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        s_abort = 0;
        for (int i = 0; i < kConvStages; ++i) {
            mbar_init(&full_bar[i], 1);
            mbar_init(&empty_bar[i], 1);
        }
        for (int i = 0; i < kConvAcc; ++i) {
            mbar_init(&accf_bar[i], 1);
            mbar_init(&acce_bar[i], 4);  // one arrival per epilogue warp
        }
        mbar_fence_init();
    }
    if (warp == 1)
        tmem_alloc(&s_tmem, kConvAcc * 16);

    // B operands: tap t as [k half][n][8 k] (core matrices of 8 n x 8 k)
    for (int i = tid; i < 27 * 16 * 16; i += kConvThreads) {
        const int t = i / 256, k = (i / 16) % 16, n = i % 16;
        const __nv_bfloat16 v = A.flip ? A.w[(26 - t) * 256 + n * 16 + k] : A.w[t * 256 + k * 16 + n];
        const int off = t * kConvTapBytes + (k / 8) * 256 + n * 16 + (k % 8) * 2;
        *reinterpret_cast<__nv_bfloat16 *>(wsm + off) = v;
    }
    fence_proxy_async_smem();
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    const uint32_t tmem = s_tmem;

    const int ntiles = A.ytiles * A.nx * A.nz;
    const int mine = ((int)blockIdx.x < ntiles) ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

    if (warp == 0) {
        // ---- producer
        int issued = 0;
        if (lane == 0) {
            for (int j = 0; j < mine; ++j) {
                const int st = j % kConvStages;
                if (j >= kConvStages &&
                    !mbar_wait_bounded(&empty_bar[st], ((j / kConvStages) - 1) & 1, &s_abort))
                    break;
                const int tile = blockIdx.x + j * gridDim.x;
                const int yt = tile % A.ytiles, rest = tile / A.ytiles;
                const int x = rest % A.nx, z = rest / A.nx;
                mbar_arrive_expect_tx(&full_bar[st], A.stage_bytes);
                if (A.hp_in)  // 18 groups of 8 voxels from y - 8
                    tma_load_5d(smem + st * kConvStageStride, &A.act, 0, yt * 16 - 1, 0, x - 1,
                                z - 1, &full_bar[st]);
                else
                    tma_load_5d(smem + st * kConvStageStride, &A.act, 0, yt * 128 - 1, 0, x - 1,
                                z - 1, &full_bar[st]);
                ++issued;
            }
            if (s_abort) {
                // drain the copies in flight of this CTA (bounded)
                volatile int drain_flag = 0;
                for (int j = issued > kConvStages ? issued - kConvStages : 0; j < issued; ++j)
                    mbar_wait_bounded(&full_bar[j % kConvStages], (j / kConvStages) & 1,
                                      (int *)&drain_flag);
            }
        }
    } else if (warp == 1) {
        // ---- MMA issue
        if (lane == 0) {
            const uint32_t idesc = umma_idesc_bf16_f32(128, 16);
            const uint32_t b0 = smem_addr(wsm);
            int done = 0;
            for (int j = 0; j < mine; ++j) {
                const int st = j % kConvStages, slot = j % kConvAcc;
                if (!mbar_wait_bounded(&full_bar[st], (j / kConvStages) & 1, &s_abort))
                    break;
                if (j >= kConvAcc &&
                    !mbar_wait_bounded(&acce_bar[slot], ((j / kConvAcc) - 1) & 1, &s_abort))
                    break;
                tc_fence_after_sync();
                const uint32_t a0 =
                    smem_addr(smem + st * kConvStageStride) + (A.vox_base - 1) * 16;
                for (int t = 0; t < 27; ++t) {
                    const int dz = t / 9, dx = (t / 3) % 3, dy = t % 3;
                    const uint32_t a = a0 + (dz * 3 + dx) * A.row_bytes + dy * 16;
                    const uint64_t ad = umma_smem_desc(a, A.half_bytes, 128);
                    const uint64_t bd = umma_smem_desc(b0 + t * kConvTapBytes, 256, 128);
                    umma_bf16(tmem + slot * 16, ad, bd, idesc, t > 0 ? 1u : 0u);
                }
                umma_commit(&empty_bar[st]);
                umma_commit(&accf_bar[slot]);
                done = j + 1;
            }
            if (s_abort && done > 0) {
                // the last committed MMAs finish before TMEM is freed (bounded)
                volatile int drain_flag = 0;
                const int j = done - 1;
                mbar_wait_bounded(&accf_bar[j % kConvAcc], (j / kConvAcc) & 1, (int *)&drain_flag);
            }
        }
    } else {
        // ---- epilogue: warp w reads TMEM lanes 32 * (w % 4) .. + 31
        const int q = warp & 3;
        float bias[16];
#pragma unroll
        for (int c = 0; c < 16; ++c)
            bias[c] = A.bias ? __ldg(A.bias + c) : 0.f;
        for (int j = 0; j < mine; ++j) {
            const int slot = j % kConvAcc;
            if (!mbar_wait_bounded(&accf_bar[slot], (j / kConvAcc) & 1, &s_abort))
                break;
            tc_fence_after_sync();
            float acc[16];
            tmem_load16(tmem + ((uint32_t)(32 * q) << 16) + slot * 16, acc);
            tc_fence_before_sync();
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&acce_bar[slot]))
                             : "memory");
            const int tile = blockIdx.x + j * gridDim.x;
            const int yt = tile % A.ytiles, rest = tile / A.ytiles;
            const int x = rest % A.nx, z = rest / A.nx;
            const int y = yt * 128 + 32 * q + lane;
            if (y < A.ny) {
                const long long v = ((long long)z * A.nx + x) * A.ny + y;
                float o[16];
#pragma unroll
                for (int c = 0; c < 16; ++c)
                    o[c] = acc[c] + bias[c];
                if (A.addend) {
                    const float4 *ap = reinterpret_cast<const float4 *>(A.addend + v * 16);
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const float4 a4 = __ldg(ap + k);
                        o[4 * k] += a4.x;
                        o[4 * k + 1] += a4.y;
                        o[4 * k + 2] += a4.z;
                        o[4 * k + 3] += a4.w;
                    }
                }
                if (A.relu) {
#pragma unroll
                    for (int c = 0; c < 16; ++c)
                        o[c] = fmaxf(o[c], 0.f);
                }
                // element offsets of the voxel's two channel halves in the input layout
                const long long zx = (long long)z * A.nx + x;
                const long long h0 = A.hp_in ? (zx * 2) * A.ypad * 8 + (long long)y * 8 : v * 16;
                const long long h1 = A.hp_in ? h0 + (long long)A.ypad * 8 : v * 16 + 8;
                if (A.mask) {
                    const uint4 m0 = __ldg(reinterpret_cast<const uint4 *>(A.mask + h0));
                    const uint4 m1 = __ldg(reinterpret_cast<const uint4 *>(A.mask + h1));
                    const __nv_bfloat16 *mb0 = reinterpret_cast<const __nv_bfloat16 *>(&m0);
                    const __nv_bfloat16 *mb1 = reinterpret_cast<const __nv_bfloat16 *>(&m1);
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        if (!(__bfloat162float(mb0[c]) > 0.f))
                            o[c] = 0.f;
                        if (!(__bfloat162float(mb1[c]) > 0.f))
                            o[8 + c] = 0.f;
                    }
                }
                if (A.out_fp32) {
                    float4 *op = reinterpret_cast<float4 *>(static_cast<float *>(A.out) + v * 16);
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        op[k] = make_float4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
                } else {
                    __align__(16) __nv_bfloat16 ob[16];
#pragma unroll
                    for (int c = 0; c < 16; ++c)
                        ob[c] = __float2bfloat16_rn(o[c]);
                    __nv_bfloat16 *ob0 = static_cast<__nv_bfloat16 *>(A.out);
                    const long long o0 = A.hp_out ? (zx * 2) * A.ypad * 8 + (long long)y * 8 : v * 16;
                    const long long o1 = A.hp_out ? o0 + (long long)A.ypad * 8 : v * 16 + 8;
                    *reinterpret_cast<uint4 *>(ob0 + o0) = reinterpret_cast<const uint4 *>(ob)[0];
                    *reinterpret_cast<uint4 *>(ob0 + o1) = reinterpret_cast<const uint4 *>(ob)[1];
                }
            }
        }
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    if (tid == 0 && s_abort)
        atomicOr(A.err, 1);
    if (warp == 1)
        tmem_dealloc(tmem, kConvAcc * 16);
}

int conv_smem_bytes() { return kConvSmem; }

cudaError_t launch_conv3_tc(EncodeTiledFn encode, const ConvLaunch &c, int num_sms,
                            cudaStream_t st, int *d_err)
{
    ConvTcArgs A;
    memset(&A, 0, sizeof A);
    // The BF16 input as (8 ch, y, half, x, z) for channels-last
    // [z][x][y][16]; half-planar [z][x][half][ypad][8] as (64 = 8 voxels x 8
    // ch, ypad/8 groups, half, x, z), whose 128-byte inner box is one burst.
    const int ypad = (c.ny + 7) / 8 * 8;
    cuuint64_t dims[5], strides[4];
    cuuint32_t box[5];
    if (c.hp_in) {
        const cuuint64_t d[5] = {64, (cuuint64_t)ypad / 8, 2, (cuuint64_t)c.nx, (cuuint64_t)c.nz};
        const cuuint64_t s[4] = {128, (cuuint64_t)16 * ypad, (cuuint64_t)32 * ypad,
                                 (cuuint64_t)32 * ypad * c.nx};
        const cuuint32_t b[5] = {64, kConvVoxHP / 8, 2, 3, 3};
        memcpy(dims, d, sizeof d);
        memcpy(strides, s, sizeof s);
        memcpy(box, b, sizeof b);
    } else {
        const cuuint64_t d[5] = {8, (cuuint64_t)c.ny, 2, (cuuint64_t)c.nx, (cuuint64_t)c.nz};
        const cuuint64_t s[4] = {32, 16, (cuuint64_t)32 * c.ny, (cuuint64_t)32 * c.ny * c.nx};
        const cuuint32_t b[5] = {8, kConvVoxCL, 2, 3, 3};
        memcpy(dims, d, sizeof d);
        memcpy(strides, s, sizeof s);
        memcpy(box, b, sizeof b);
    }
    cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    CUresult r = encode(&A.act, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void *>(c.x), dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    A.w = static_cast<const __nv_bfloat16 *>(c.w);
    A.bias = c.bias;
    A.mask = static_cast<const __nv_bfloat16 *>(c.mask);
    A.addend = c.addend;
    A.out = c.y;
    A.err = d_err;
    A.ny = c.ny;
    A.nx = c.nx;
    A.nz = c.nz;
    A.ytiles = (c.ny + 127) / 128;
    A.relu = c.relu;
    A.out_fp32 = c.out_fp32;
    A.flip = c.flip;
    A.hp_in = c.hp_in;
    A.hp_out = c.hp_out;
    A.ypad = ypad;
    const int vox = c.hp_in ? kConvVoxHP : kConvVoxCL;
    A.half_bytes = vox * 16;
    A.row_bytes = 2 * vox * 16;
    A.stage_bytes = kConvRows * A.row_bytes;
    A.vox_base = c.hp_in ? 8 : 1;
    cudaError_t e = cudaFuncSetAttribute(conv3_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kConvSmem);
    if (e != cudaSuccess)
        return e;
    const int tiles = A.ytiles * c.nx * c.nz;
    const int grid = tiles < num_sms ? tiles : num_sms;
    conv3_tc_kernel<<<grid, kConvThreads, kConvSmem, st>>>(A);
    return cudaGetLastError();
}

}  // namespace asets
