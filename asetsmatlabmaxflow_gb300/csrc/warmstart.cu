// Learned warm start: the convolution entry point and (below) the small
// network that maps (Ct, alpha) to an initial (u, ps, pt).
#include <cuda_bf16.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "asets.h"
#include "internal.h"
#include "wgrad_tc.cuh"

using namespace asets;

static asets_status ws_fail(asets_status s, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    set_last_error(buf);
    return s;
}

#define WS_TRY(call)                                                                         \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            cudaGetLastError();                                                              \
            return ws_fail(e_ == cudaErrorMemoryAllocation ? ASETS_ERR_OUT_OF_MEMORY        \
                                                           : ASETS_ERR_CUDA,                 \
                           "%s: %s", #call, cudaGetErrorString(e_));                         \
        }                                                                                    \
    } while (0)

extern "C" ASETS_API asets_status asets_conv3d_bf16(asets_context *ctx, const void *x,
                                                    const void *w, const float *bias,
                                                    const void *mask, void *y, int Ny, int Nx,
                                                    int Nz, int relu, int out_fp32, int flip)
{
    if (!ctx || !x || !w || !y || Ny < 1 || Nx < 1 || Nz < 1)
        return ws_fail(ASETS_ERR_INVALID_ARG, "bad convolution arguments");
    if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15)
        return ws_fail(ASETS_ERR_INVALID_ARG, "activations must be 16-byte aligned");
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(context_device(ctx));
    int *d_err = nullptr;
    asets_status st = ASETS_OK;
    ConvLaunch c;
    c.x = x;
    c.w = w;
    c.bias = bias;
    c.mask = mask;
    c.y = y;
    c.ny = Ny;
    c.nx = Nx;
    c.nz = Nz;
    c.relu = relu;
    c.out_fp32 = out_fp32;
    c.flip = flip;
    cudaError_t e = cudaMallocAsync(&d_err, sizeof(int), context_stream(ctx));
    if (e == cudaSuccess)
        e = cudaMemsetAsync(d_err, 0, sizeof(int), context_stream(ctx));
    if (e == cudaSuccess)
        e = launch_conv3_tc(context_encoder(ctx), c, context_num_sms(ctx), context_stream(ctx),
                            d_err);
    int herr = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, context_stream(ctx));
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(context_stream(ctx));
    if (d_err)
        cudaFreeAsync(d_err, context_stream(ctx));
    if (e != cudaSuccess) {
        cudaGetLastError();
        st = ws_fail(ASETS_ERR_CUDA, "convolution: %s", cudaGetErrorString(e));
    } else if (herr) {
        st = ws_fail(ASETS_ERR_TIMEOUT, "convolution: a device-side wait timed out");
    }
    cudaSetDevice(prev);
    return st;
}

// ===================================================================== net
// Four 3x3x3 convolutional layers, 16 hidden channels, ReLU between them:
//   input   (Ct_1..Ct_L, alpha)                                channels 0..L
//   output  (u_1..u_L, ps, pt_1..pt_L, bx_1..bx_L/alpha, by_1..by_L/alpha,
//            bz_1..bz_L/alpha)                                 channels 0..5L
// The last layer has 32 output channels, computed as two 16-channel blocks
// (parameter blocks 3 and 4) from the same input.  The spatial flows are
// predicted relative to alpha (the projection keeps |p| <= alpha).  Weights
// are kept in FP32 (the Adam master copy) and used as BF16.
namespace {

constexpr int kBlocks = 5;        // 3 hidden layers + 2 output halves
constexpr int kW = 27 * 16 * 16;  // weights of one block
constexpr int kParams = kBlocks * (kW + 16);
constexpr int kOut = 32;          // output channels (two blocks of 16)

// (Ct_1..Ct_L, alpha) -> the BF16 input of the first layer, half-planar
// ([z][x][half][ypad][8], the layout of every BF16 activation of the net).
__global__ void pack_input_kernel(const float *ct, const float *alpha, __nv_bfloat16 *x,
                                  long long n, int L, int ny)
{
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
         g += (long long)gridDim.x * blockDim.x) {
        __align__(16) __nv_bfloat16 v[16];
        for (int c = 0; c < 16; ++c) {
            float f = 0.f;
            if (c < L)
                f = ct[c * n + g];
            else if (c == L)
                f = alpha[g];
            v[c] = __float2bfloat16_rn(f);
        }
        const long long zx = g / ny, y = g % ny, yp = (ny + 7) / 8 * 8;
        *reinterpret_cast<uint4 *>(x + (zx * 2) * yp * 8 + y * 8) = reinterpret_cast<const uint4 *>(v)[0];
        *reinterpret_cast<uint4 *>(x + (zx * 2 + 1) * yp * 8 + y * 8) =
            reinterpret_cast<const uint4 *>(v)[1];
    }
}

// Output channel c of voxel g in the [2][n][16] output/target layout.
__device__ __forceinline__ long long out_index(int c, long long g, long long n)
{
    return (c >> 4) * n * 16 + g * 16 + (c & 15);
}

struct NetIO {
    const float *alpha;
    float *u, *ps, *pt, *bx, *by, *bz;  // Matlab layout, label slowest
};

__global__ void pack_target_kernel(NetIO io, float *t, long long n, int L)
{
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
         g += (long long)gridDim.x * blockDim.x) {
        const float ia = 1.f / io.alpha[g];
        for (int c = 0; c < kOut; ++c) {
            float f = 0.f;
            if (c < L)
                f = io.u[c * n + g];
            else if (c == L)
                f = io.ps[g];
            else if (c <= 2 * L)
                f = io.pt[(c - L - 1) * n + g];
            else if (c <= 5 * L) {
                const int k = c - 2 * L - 1, axis = k / L, l = k % L;
                const float *b = axis == 0 ? io.bx : (axis == 1 ? io.by : io.bz);
                f = b[l * n + g] * ia;
            }
            t[out_index(c, g, n)] = f;
        }
    }
}

__global__ void unpack_output_kernel(const float *out, NetIO io, long long n, int L)
{
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
         g += (long long)gridDim.x * blockDim.x) {
        for (int l = 0; l < L; ++l) {
            io.u[l * n + g] = fminf(fmaxf(out[out_index(l, g, n)], 0.f), 1.f);  // u in [0, 1]
            io.pt[l * n + g] = out[out_index(L + 1 + l, g, n)];
        }
        io.ps[g] = out[out_index(L, g, n)];
        if (io.bx) {
            const float a = io.alpha[g];
            for (int k = 0; k < 3 * L; ++k) {
                const int axis = k / L, l = k % L;
                float *b = axis == 0 ? io.bx : (axis == 1 ? io.by : io.bz);
                if (b)
                    b[l * n + g] = out[out_index(2 * L + 1 + k, g, n)] * a;
            }
        }
    }
}

// Mean squared error over the 5L+1 used output channels; writes the
// gradient w.r.t. the output (BF16, per 16-channel block half-planar like
// the activations: [2][z][x][half][ypad][8]) and accumulates the loss.
__global__ void loss_kernel(const float *out, const float *tgt, __nv_bfloat16 *g, long long n,
                            int used, float scale, float *loss, int ny)
{
    float acc = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < 2 * n * 16;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)((i / (n * 16)) * 16 + (i & 15));
        float d = 0.f;
        if (c < used) {
            d = out[i] - tgt[i];
            acc += d * d;
        }
        const long long blk = i / (n * 16), v = (i / 16) % n, cc = i & 15;
        const long long zx = v / ny, y = v % ny, yp = (ny + 7) / 8 * 8;
        const long long pn = yp * (n / ny);  // padded voxels of one 16-channel block
        g[blk * pn * 16 + (zx * 2 + cc / 8) * yp * 8 + y * 8 + (cc & 7)] =
            __float2bfloat16_rn(2.f * d * scale);
    }
    for (int o = 16; o > 0; o >>= 1)
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0)
        atomicAdd(loss, acc * scale);
}

// Adam on the FP32 master parameters; clears the gradients.
__global__ void adam_kernel(float *p, float *m, float *v, float *grad, int n, float lr, float b1,
                            float b2, float eps, float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = grad[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        grad[i] = 0.f;
    }
}

// BF16 copies of the weights (parameter block b: kW weights then 16 biases).
__global__ void to_bf16_kernel(const float *p, __nv_bfloat16 *w16)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kBlocks * kW;
         i += gridDim.x * blockDim.x) {
        const int b = i / kW, j = i % kW;
        w16[i] = __float2bfloat16_rn(p[b * (kW + 16) + j]);
    }
}

int blocks_for(long long n, int threads, int num_sms)
{
    long long b = (n + threads - 1) / threads;
    long long cap = (long long)num_sms * 8;
    return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

}  // namespace

struct asets_wsnet {
    asets_context *ctx = nullptr;
    int L = 6;
    float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *w16 = nullptr;
    float *loss = nullptr;
    int *err = nullptr;
    long long vox_cap = 0, pvox_cap = 0;
    int shape[3] = {0, 0, 0};         // volume the half-planar padding was cleared for
    __nv_bfloat16 *x0 = nullptr, *act[3] = {nullptr, nullptr, nullptr};
    __nv_bfloat16 *gbuf[2] = {nullptr, nullptr};  // [v][16] gradients of hidden layers
    __nv_bfloat16 *gout = nullptr;                // [2][v][16] gradient of the output
    float *out = nullptr, *tgt = nullptr;         // [2][v][16]
    float *part = nullptr;                        // [v][16] first half of a summed dgrad
    float *wg_partial = nullptr;                  // [SMs][28][16][16] weight-gradient partials
    int step = 0;
};

// Buffers for a Ny x Nx x Nz volume.  The BF16 activations and gradients
// are half-planar with rows padded to ypad = Ny rounded up to 8 voxels
// (pvox = ypad * Nx * Nz per 16-channel block); the convolutions read the
// padding, so it must be zero: every buffer is cleared when the shape
// changes (the kernels write real voxels only).
static asets_status ws_reserve(asets_wsnet *n, int Ny, int Nx, int Nz)
{
    const long long vox = (long long)Ny * Nx * Nz;
    const long long pvox = (long long)((Ny + 7) / 8 * 8) * Nx * Nz;
    cudaStream_t st = context_stream(n->ctx);
    const bool same = (Ny == n->shape[0] && Nx == n->shape[1] && Nz == n->shape[2]);
    if (vox <= n->vox_cap && pvox <= n->pvox_cap) {
        if (!same) {
            __nv_bfloat16 *hp[] = {n->x0, n->act[0], n->act[1], n->act[2], n->gbuf[0], n->gbuf[1]};
            for (__nv_bfloat16 *b : hp)
                WS_TRY(cudaMemsetAsync(b, 0, (size_t)pvox * 32, st));
            WS_TRY(cudaMemsetAsync(n->gout, 0, (size_t)pvox * 64, st));
            n->shape[0] = Ny;
            n->shape[1] = Nx;
            n->shape[2] = Nz;
        }
        return ASETS_OK;
    }
    void **bufs[] = {(void **)&n->x0,      (void **)&n->act[0], (void **)&n->act[1],
                     (void **)&n->act[2],  (void **)&n->gbuf[0], (void **)&n->gbuf[1],
                     (void **)&n->gout,    (void **)&n->out,    (void **)&n->tgt,
                     (void **)&n->part};
    for (void **b : bufs)
        if (*b) {
            cudaFreeAsync(*b, st);
            *b = nullptr;
        }
    n->vox_cap = 0;
    n->pvox_cap = 0;
    const size_t b16 = (size_t)pvox * 16 * sizeof(__nv_bfloat16), f32 = (size_t)vox * 16 * 4;
    const size_t sizes[] = {b16, b16, b16, b16, b16, b16, 2 * b16, 2 * f32, 2 * f32, f32};
    for (int i = 0; i < 10; ++i) {
        WS_TRY(cudaMallocAsync(bufs[i], sizes[i], st));
        if (i < 7)
            WS_TRY(cudaMemsetAsync(*bufs[i], 0, sizes[i], st));
    }
    n->vox_cap = vox;
    n->pvox_cap = pvox;
    n->shape[0] = Ny;
    n->shape[1] = Nx;
    n->shape[2] = Nz;
    return ASETS_OK;
}

extern "C" ASETS_API int asets_wsnet_num_params(void) { return kParams; }

extern "C" ASETS_API asets_status asets_wsnet_create(asets_context *ctx, int nLab,
                                                     unsigned long long seed, asets_wsnet **out)
{
    if (!ctx || !out || nLab < 1 || 5 * nLab + 1 > kOut)
        return ws_fail(ASETS_ERR_INVALID_ARG, "warm-start net needs 1 <= nLab <= 6");
    *out = nullptr;
    cudaSetDevice(context_device(ctx));
    asets_wsnet *n = new asets_wsnet;
    n->ctx = ctx;
    n->L = nLab;
    cudaStream_t st = context_stream(ctx);
    auto fail_free = [&](asets_status s) {
        asets_wsnet_destroy(n);
        return s;
    };
    float **pbufs[] = {&n->params, &n->grads, &n->m, &n->v};
    for (float **b : pbufs)
        if (cudaMallocAsync((void **)b, kParams * 4, st) != cudaSuccess)
            return fail_free(ws_fail(ASETS_ERR_OUT_OF_MEMORY, "warm-start net: out of memory"));
    if (cudaMallocAsync((void **)&n->w16, kBlocks * kW * 2, st) != cudaSuccess ||
        cudaMallocAsync((void **)&n->loss, 4, st) != cudaSuccess ||
        cudaMallocAsync((void **)&n->err, 4, st) != cudaSuccess ||
        cudaMallocAsync((void **)&n->wg_partial,
                        (size_t)context_num_sms(ctx) * kWgtTaps * 256 * sizeof(float), st) !=
            cudaSuccess)
        return fail_free(ws_fail(ASETS_ERR_OUT_OF_MEMORY, "warm-start net: out of memory"));
    // He-normal initial weights from a seeded generator (Box-Muller on a
    // 64-bit LCG), zero biases; weights of unused channels stay zero.
    std::vector<float> h(kParams, 0.f);
    unsigned long long s = seed * 6364136223846793005ull + 1442695040888963407ull;
    auto uni = [&]() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return ((s >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    const int used = 5 * nLab + 1;
    for (int b = 0; b < kBlocks; ++b) {
        const int cin = (b == 0) ? nLab + 1 : 16;
        int cout = 16;
        if (b == 3)
            cout = used < 16 ? used : 16;
        else if (b == 4)
            cout = used > 16 ? used - 16 : 0;
        const double sd = sqrt(2.0 / (27.0 * cin));
        for (int t = 0; t < 27; ++t)
            for (int i = 0; i < cin; ++i)
                for (int o = 0; o < cout; ++o) {
                    const double r = sqrt(-2.0 * log(uni())) * cos(6.283185307179586 * uni());
                    h[b * (kW + 16) + (t * 16 + i) * 16 + o] = (float)((b >= 3 ? 0.5 : 1.0) * sd * r);
                }
    }
    if (cudaMemcpyAsync(n->params, h.data(), kParams * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(n->grads, 0, kParams * 4, st) != cudaSuccess ||
        cudaMemsetAsync(n->m, 0, kParams * 4, st) != cudaSuccess ||
        cudaMemsetAsync(n->v, 0, kParams * 4, st) != cudaSuccess)
        return fail_free(ws_fail(ASETS_ERR_CUDA, "warm-start net: initialisation copy failed"));
    to_bf16_kernel<<<64, 256, 0, st>>>(n->params, n->w16);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
        return fail_free(ws_fail(ASETS_ERR_CUDA, "warm-start net: initialisation failed"));
    *out = n;
    return ASETS_OK;
}

extern "C" ASETS_API void asets_wsnet_destroy(asets_wsnet *n)
{
    if (!n)
        return;
    cudaStream_t st = context_stream(n->ctx);
    void *ps[] = {n->params, n->grads,   n->m,       n->v,    n->w16,  n->loss,
                  n->err,    n->x0,      n->act[0],  n->act[1], n->act[2], n->gbuf[0],
                  n->gbuf[1], n->gout,   n->out,     n->tgt,  n->part, n->wg_partial};
    for (void *p : ps)
        if (p)
            cudaFreeAsync(p, st);
    cudaStreamSynchronize(st);
    delete n;
}

extern "C" ASETS_API asets_status asets_wsnet_get_params(asets_wsnet *n, float *host)
{
    if (!n || !host)
        return ws_fail(ASETS_ERR_INVALID_ARG, "NULL argument");
    WS_TRY(cudaMemcpyAsync(host, n->params, kParams * 4, cudaMemcpyDeviceToHost, context_stream(n->ctx)));
    WS_TRY(cudaStreamSynchronize(context_stream(n->ctx)));
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_wsnet_set_params(asets_wsnet *n, const float *host)
{
    if (!n || !host)
        return ws_fail(ASETS_ERR_INVALID_ARG, "NULL argument");
    cudaStream_t st = context_stream(n->ctx);
    WS_TRY(cudaMemcpyAsync(n->params, host, kParams * 4, cudaMemcpyHostToDevice, st));
    to_bf16_kernel<<<64, 256, 0, st>>>(n->params, n->w16);
    WS_TRY(cudaGetLastError());
    n->step = 0;
    WS_TRY(cudaMemsetAsync(n->m, 0, kParams * 4, st));
    WS_TRY(cudaMemsetAsync(n->v, 0, kParams * 4, st));
    WS_TRY(cudaStreamSynchronize(st));
    return ASETS_OK;
}

static ConvLaunch conv_of(asets_wsnet *n, int b, const void *x, void *y, int Ny, int Nx, int Nz)
{
    ConvLaunch c{};
    c.x = x;
    c.w = n->w16 + (size_t)b * kW;
    c.y = y;
    c.ny = Ny;
    c.nx = Nx;
    c.nz = Nz;
    c.hp_in = 1;   // the net's BF16 activations are half-planar
    c.hp_out = 1;
    return c;
}

// Forward pass: x0 -> act[0..2] -> out (FP32, two 16-channel halves).
static asets_status ws_forward(asets_wsnet *n, int Ny, int Nx, int Nz, const float *ct,
                               const float *alpha)
{
    const long long vox = (long long)Ny * Nx * Nz;
    asets_status s = ws_reserve(n, Ny, Nx, Nz);
    if (s != ASETS_OK)
        return s;
    cudaStream_t st = context_stream(n->ctx);
    const int sms = context_num_sms(n->ctx);
    EncodeTiledFn enc = context_encoder(n->ctx);
    pack_input_kernel<<<blocks_for(vox, 256, sms), 256, 0, st>>>(ct, alpha, n->x0, vox, n->L, Ny);
    WS_TRY(cudaGetLastError());
    WS_TRY(cudaMemsetAsync(n->err, 0, 4, st));
    const void *in = n->x0;
    for (int b = 0; b < kBlocks; ++b) {
        void *y = b < 3 ? static_cast<void *>(n->act[b])
                        : static_cast<void *>(n->out + (size_t)(b - 3) * vox * 16);
        ConvLaunch c = conv_of(n, b, in, y, Ny, Nx, Nz);
        c.bias = n->params + (size_t)b * (kW + 16) + kW;
        c.relu = b < 3 ? 1 : 0;
        c.out_fp32 = b < 3 ? 0 : 1;
        WS_TRY(launch_conv3_tc(enc, c, sms, st, n->err));
        if (b < 3)
            in = y;
    }
    return ASETS_OK;
}

static asets_status ws_check(asets_wsnet *n)
{
    int herr = 0;
    WS_TRY(cudaMemcpyAsync(&herr, n->err, 4, cudaMemcpyDeviceToHost, context_stream(n->ctx)));
    WS_TRY(cudaStreamSynchronize(context_stream(n->ctx)));
    if (herr)
        return ws_fail(ASETS_ERR_TIMEOUT, "a device-side wait timed out in the warm-start net");
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_wsnet_predict(asets_wsnet *n, int Ny, int Nx, int Nz,
                                                      const float *Ct, const float *alpha,
                                                      float *u0, float *ps0, float *pt0,
                                                      float *bx0, float *by0, float *bz0)
{
    if (!n || !Ct || !alpha || !u0 || !ps0 || !pt0 || Ny < 1 || Nx < 1 || Nz < 1)
        return ws_fail(ASETS_ERR_INVALID_ARG, "bad arguments");
    if ((bx0 || by0 || bz0) && !(bx0 && by0 && bz0))
        return ws_fail(ASETS_ERR_INVALID_ARG, "initial flows need bx0, by0 and bz0 (or none)");
    cudaSetDevice(context_device(n->ctx));
    asets_status s = ws_forward(n, Ny, Nx, Nz, Ct, alpha);
    if (s != ASETS_OK)
        return s;
    const long long vox = (long long)Ny * Nx * Nz;
    cudaStream_t st = context_stream(n->ctx);
    NetIO io{alpha, u0, ps0, pt0, bx0, by0, bz0};
    unpack_output_kernel<<<blocks_for(vox, 256, context_num_sms(n->ctx)), 256, 0, st>>>(
        n->out, io, vox, n->L);
    WS_TRY(cudaGetLastError());
    return ws_check(n);
}

// Forward + backward; gradients accumulate into n->grads.
static asets_status ws_backward(asets_wsnet *n, int Ny, int Nx, int Nz, const float *ct,
                                const float *alpha, const NetIO &target, float *loss_out)
{
    asets_status s = ws_forward(n, Ny, Nx, Nz, ct, alpha);
    if (s != ASETS_OK)
        return s;
    const long long vox = (long long)Ny * Nx * Nz;
    const long long pvox = (long long)((Ny + 7) / 8 * 8) * Nx * Nz;  // a padded half-planar block
    cudaStream_t st = context_stream(n->ctx);
    const int sms = context_num_sms(n->ctx);
    EncodeTiledFn enc = context_encoder(n->ctx);
    pack_target_kernel<<<blocks_for(vox, 256, sms), 256, 0, st>>>(target, n->tgt, vox, n->L);
    WS_TRY(cudaMemsetAsync(n->loss, 0, 4, st));
    const int used = 5 * n->L + 1;
    const float scale = 1.0f / (float)((double)vox * used);
    loss_kernel<<<blocks_for(vox * 32, 256, sms), 256, 0, st>>>(n->out, n->tgt, n->gout, vox, used,
                                                                scale, n->loss, Ny);
    WS_TRY(cudaGetLastError());
    // output blocks 3 and 4: weight gradients, then the data gradient
    // flip(g3, W3) + flip(g4, W4), masked by the ReLU of act[2]
    for (int b = 3; b < kBlocks; ++b) {
        float *gw = n->grads + (size_t)b * (kW + 16);
        WS_TRY(launch_wgrad_tc(enc, n->act[2], n->gout + (size_t)(b - 3) * pvox * 16, gw, gw + kW,
                               Ny, Nx, Nz, n->wg_partial, sms, n->err, st, 1));
    }
    {
        ConvLaunch c = conv_of(n, 3, n->gout, n->part, Ny, Nx, Nz);
        c.flip = 1;
        c.out_fp32 = 1;
        WS_TRY(launch_conv3_tc(enc, c, sms, st, n->err));
        ConvLaunch d = conv_of(n, 4, n->gout + (size_t)pvox * 16, n->gbuf[0], Ny, Nx, Nz);
        d.flip = 1;
        d.addend = n->part;
        d.mask = n->act[2];
        WS_TRY(launch_conv3_tc(enc, d, sms, st, n->err));
    }
    // hidden layers 2, 1, 0: input activation and the gradient w.r.t. the output
    const __nv_bfloat16 *ins[3] = {n->x0, n->act[0], n->act[1]};
    int cur = 0;
    for (int l = 2; l >= 0; --l) {
        float *gw = n->grads + (size_t)l * (kW + 16);
        WS_TRY(launch_wgrad_tc(enc, ins[l], n->gbuf[cur], gw, gw + kW, Ny, Nx, Nz, n->wg_partial,
                               sms, n->err, st, 1));
        if (l == 0)
            break;
        ConvLaunch c = conv_of(n, l, n->gbuf[cur], n->gbuf[cur ^ 1], Ny, Nx, Nz);
        c.mask = ins[l];  // ReLU of the layer below: its output is this layer's input
        c.flip = 1;
        WS_TRY(launch_conv3_tc(enc, c, sms, st, n->err));
        cur ^= 1;
    }
    s = ws_check(n);
    if (s != ASETS_OK)
        return s;
    if (loss_out) {
        WS_TRY(cudaMemcpyAsync(loss_out, n->loss, 4, cudaMemcpyDeviceToHost, st));
        WS_TRY(cudaStreamSynchronize(st));
    }
    return ASETS_OK;
}

static bool target_ok(const float *Ct, const float *alpha, const float *u, const float *ps,
                      const float *pt, const float *bx, const float *by, const float *bz)
{
    return Ct && alpha && u && ps && pt && bx && by && bz;
}

extern "C" ASETS_API asets_status asets_wsnet_gradients(asets_wsnet *n, int Ny, int Nx, int Nz,
                                                        const float *Ct, const float *alpha,
                                                        const float *u, const float *ps,
                                                        const float *pt, const float *bx,
                                                        const float *by, const float *bz,
                                                        float *host_grads, float *loss)
{
    if (!n || !target_ok(Ct, alpha, u, ps, pt, bx, by, bz) || !host_grads || Ny < 1 || Nx < 1 ||
        Nz < 1)
        return ws_fail(ASETS_ERR_INVALID_ARG, "bad arguments");
    cudaSetDevice(context_device(n->ctx));
    cudaStream_t st = context_stream(n->ctx);
    WS_TRY(cudaMemsetAsync(n->grads, 0, kParams * 4, st));
    NetIO tgt{alpha, const_cast<float *>(u), const_cast<float *>(ps), const_cast<float *>(pt),
              const_cast<float *>(bx), const_cast<float *>(by), const_cast<float *>(bz)};
    asets_status s = ws_backward(n, Ny, Nx, Nz, Ct, alpha, tgt, loss);
    if (s != ASETS_OK)
        return s;
    WS_TRY(cudaMemcpyAsync(host_grads, n->grads, kParams * 4, cudaMemcpyDeviceToHost, st));
    WS_TRY(cudaMemsetAsync(n->grads, 0, kParams * 4, st));
    WS_TRY(cudaStreamSynchronize(st));
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_wsnet_train_step(asets_wsnet *n, int Ny, int Nx, int Nz,
                                                         const float *Ct, const float *alpha,
                                                         const float *u, const float *ps,
                                                         const float *pt, const float *bx,
                                                         const float *by, const float *bz,
                                                         float lr, float *loss)
{
    if (!n || !target_ok(Ct, alpha, u, ps, pt, bx, by, bz) || Ny < 1 || Nx < 1 || Nz < 1)
        return ws_fail(ASETS_ERR_INVALID_ARG, "bad arguments");
    cudaSetDevice(context_device(n->ctx));
    NetIO tgt{alpha, const_cast<float *>(u), const_cast<float *>(ps), const_cast<float *>(pt),
              const_cast<float *>(bx), const_cast<float *>(by), const_cast<float *>(bz)};
    asets_status s = ws_backward(n, Ny, Nx, Nz, Ct, alpha, tgt, loss);
    if (s != ASETS_OK)
        return s;
    n->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)n->step), c2 = 1.f - powf(b2, (float)n->step);
    cudaStream_t st = context_stream(n->ctx);
    adam_kernel<<<64, 256, 0, st>>>(n->params, n->m, n->v, n->grads, kParams, lr, b1, b2, 1e-8f,
                                    c1, c2);
    to_bf16_kernel<<<64, 256, 0, st>>>(n->params, n->w16);
    WS_TRY(cudaGetLastError());
    return ASETS_OK;
}
