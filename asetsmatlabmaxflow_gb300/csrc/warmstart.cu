// Learned warm start: the convolution entry point and (below) the small
// network that maps (Ct, alpha) to an initial (u, ps, pt).
#include <cuda_bf16.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "asets.h"
#include "internal.h"

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
