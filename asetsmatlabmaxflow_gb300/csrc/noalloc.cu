// Allocation-free binary 3D solve.
//
// Some callers cannot allocate device memory at solve time: a host
// application whose device memory is owned by another allocator (a framework
// with a caching allocator that has reserved the GPU, or Matlab's gpuArray
// memory manager around a mex file), or a long-running pipeline that sizes
// and reserves everything at start-up and forbids allocation afterwards.
// For them asets_binary_mf3d_noalloc() runs the same fused iteration kernel as
// asets_binary_mf3d() but takes every input and output as a device pointer and
// keeps all of its scratch -- padded inputs, the ping-pong flow and
// ps/pt/u state, the iteration control block and the erriter partials -- in
// one file-scope device array of fixed size.  It calls no cudaMalloc,
// cudaFree or other allocating routine.
//
// That array (kNoallocScratchBytes, about 15 MiB) is device memory of the
// library's module: with CUDA's lazy module loading (the default) it is
// reserved when the first call on a device looks up its address, and at
// library load with CUDA_MODULE_LOADING=EAGER; from then on the device holds
// it until the process exits.  A caller that hands the GPU to another
// allocator makes one small call first (a 1 x 1 x 1 problem with maxIt 0
// will do).  Problems whose padded volume exceeds kNoallocMaxCells voxels
// are rejected.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "asets.h"
#include "internal.h"

using namespace asets;

namespace {

constexpr long long kNoallocMaxCells = 262144;  // padded voxels (row pitch x Nx x Nz)
constexpr size_t kFieldBytes = (size_t)kNoallocMaxCells * sizeof(float);
// 3 inputs + 2 parities x (3 flow components + ps + pt + u)
constexpr size_t kNumFields = 3 + 2 * 6;
constexpr size_t kControlBytes = 256;
constexpr int kMaxBlocks = 1024;
constexpr int kMaxItems = 16384;              // work items of one launch
constexpr size_t kDescBytes = (sizeof(ProblemDesc) + 255) / 256 * 256;
constexpr size_t kQueueBytes = 256;
constexpr size_t kItemBytes = kMaxItems * (sizeof(int) + sizeof(double));
constexpr size_t kNoallocScratchBytes =
    kNumFields * kFieldBytes + kControlBytes + kDescBytes + kQueueBytes + kItemBytes;
constexpr int kLaunchChunk = 64;              // iterations queued between done-flag reads

}  // namespace

// The scratch of every call on this device.  In host code this name is only
// a host-side stand-in; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

namespace {

typedef CUresult (*PFN_encodeTiled_na)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                      const cuuint64_t *, const cuuint64_t *,
                                      const cuuint32_t *, const cuuint32_t *,
                                      CUtensorMapInterleave, CUtensorMapSwizzle,
                                      CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

struct DeviceSetup {
    bool ready = false;
    unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch
    int num_sms = 0;
    PFN_encodeTiled_na encode = nullptr;
    std::mutex call_mu;                // serialises calls on this device
};

constexpr int kMaxDevices = 64;
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

// Reset of the control block for a new solve, on the solve's stream.
__global__ void noalloc_reset_kernel(IterControl *ctl, int max_it, float err_bound, float denom)
{
    IterControl c;
    memset(&c, 0, sizeof c);
    c.done = (max_it == 0) ? 1 : 0;
    c.last_iter = -1;
    c.max_it = max_it;
    c.err_bound = err_bound;
    c.break_lt = 0;
    c.denom = denom;
    *ctl = c;
}

asets_status na_fail(asets_status s, const char *fmt, ...)
{
    static thread_local char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    set_last_error(buf);
    return s;
}

// Set-up once per device, with that device current: look up the scratch
// array's device address and the driver's tensor-map encoder.
asets_status setup_device(int dev, DeviceSetup **out)
{
    if (dev < 0 || dev >= kMaxDevices)
        return na_fail(ASETS_ERR_UNSUPPORTED, "device index %d not supported", dev);
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSetup &d = g_setup[dev];
    if (!d.ready) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            // the lookup loads the module, which reserves the array
            return na_fail(e == cudaErrorMemoryAllocation ? ASETS_ERR_OUT_OF_MEMORY
                                                          : ASETS_ERR_CUDA,
                           "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        }
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess)
            return na_fail(ASETS_ERR_CUDA, "cudaDeviceGetAttribute: %s", cudaGetErrorString(e));
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                             cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
            return na_fail(ASETS_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        d.scratch = static_cast<unsigned char *>(ptr);
        d.num_sms = sms;
        d.encode = reinterpret_cast<PFN_encodeTiled_na>(fn);
        d.ready = true;
    }
    *out = &d;
    return ASETS_OK;
}

asets_status noalloc_solve(DeviceSetup &dv, const asets_options *opt, const float *alpha,
                           const float *Cs, const float *Ct, int Nx, int Ny, int Nz,
                           long long pitch, long long cells, int maxIt, float errBound, float cc,
                           float steps, float *u, float *cvg, int *itNum, cudaStream_t sm);

}  // namespace

extern "C" ASETS_API asets_status asets_binary_mf3d_noalloc(
    const asets_options *opt, const float *alpha, const float *Cs, const float *Ct, int Nx,
    int Ny, int Nz, int maxIt, float errBound, float cc, float steps, float *u, float *cvg,
    int *itNum, void *stream)
{
    if (!alpha || !Cs || !Ct || !u || !itNum || (maxIt > 0 && !cvg))
        return na_fail(ASETS_ERR_INVALID_ARG, "NULL pointer argument");
    if (Nx < 1 || Ny < 1 || Nz < 1 || maxIt < 0)
        return na_fail(ASETS_ERR_INVALID_ARG, "bad sizes %d x %d x %d or maxIt %d", Ny, Nx, Nz,
                       maxIt);
    const long long pitch = (Ny >= 32) ? ((long long)Ny + 31) / 32 * 32 : ((long long)Ny + 3) / 4 * 4;
    const long long cells = pitch * Nx * Nz;
    if (cells > kNoallocMaxCells)
        return na_fail(ASETS_ERR_INVALID_ARG,
                       "problem needs %lld padded voxels; the allocation-free entry point is "
                       "limited to %lld",
                       cells, kNoallocMaxCells);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return na_fail(ASETS_ERR_NO_DEVICE, "no current CUDA device");
    }
    DeviceSetup *d = nullptr;
    asets_status st = setup_device(dev, &d);
    if (st != ASETS_OK)
        return st;
    std::lock_guard<std::mutex> call_lock(d->call_mu);
    cudaStream_t sm = static_cast<cudaStream_t>(stream);
    st = noalloc_solve(*d, opt, alpha, Cs, Ct, Nx, Ny, Nz, pitch, cells, maxIt, errBound, cc,
                       steps, u, cvg, itNum, sm);
    if (st != ASETS_OK) {
        // An error may leave this call's copies and kernels queued: let them
        // finish before the next call reuses the scratch.
        cudaStreamSynchronize(sm);
        cudaGetLastError();
    }
    return st;
}

namespace {

asets_status noalloc_solve(DeviceSetup &dv, const asets_options *opt, const float *alpha,
                           const float *Cs, const float *Ct, int Nx, int Ny, int Nz,
                           long long pitch, long long cells, int maxIt, float errBound, float cc,
                           float steps, float *u, float *cvg, int *itNum, cudaStream_t sm)
{
    DeviceSetup *d = &dv;
    // carve the scratch
    unsigned char *base = d->scratch;
    auto field = [&](int i) { return reinterpret_cast<float *>(base + (size_t)i * kFieldBytes); };
    float *cs = field(0), *ct = field(1), *al = field(2);
    float *b[2][3], *ps[2], *pt[2], *uu[2];
    for (int par = 0; par < 2; ++par) {
        for (int k = 0; k < 3; ++k)
            b[par][k] = field(3 + par * 6 + k);
        ps[par] = field(3 + par * 6 + 3);
        pt[par] = field(3 + par * 6 + 4);
        uu[par] = field(3 + par * 6 + 5);
    }
    unsigned char *tail = base + kNumFields * kFieldBytes;
    IterControl *ctl = reinterpret_cast<IterControl *>(tail);
    ProblemDesc *d_desc = reinterpret_cast<ProblemDesc *>(tail + kControlBytes);
    unsigned int *queue = reinterpret_cast<unsigned int *>(tail + kControlBytes + kDescBytes);
    double *item_partials =
        reinterpret_cast<double *>(tail + kControlBytes + kDescBytes + kQueueBytes);
    int *item_problem = reinterpret_cast<int *>(tail + kControlBytes + kDescBytes + kQueueBytes +
                                                kMaxItems * sizeof(double));

#define NA_TRY(call)                                                                     \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            cudaGetLastError();                                                          \
            return na_fail(ASETS_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));      \
        }                                                                                \
    } while (0)

    // inputs into the padded layout (device to device)
    const size_t rows = (size_t)Nx * Nz;
    NA_TRY(cudaMemcpy2DAsync(cs, pitch * 4, Cs, (size_t)Ny * 4, (size_t)Ny * 4, rows,
                             cudaMemcpyDeviceToDevice, sm));
    NA_TRY(cudaMemcpy2DAsync(ct, pitch * 4, Ct, (size_t)Ny * 4, (size_t)Ny * 4, rows,
                             cudaMemcpyDeviceToDevice, sm));
    NA_TRY(cudaMemcpy2DAsync(al, pitch * 4, alpha, (size_t)Ny * 4, (size_t)Ny * 4, rows,
                             cudaMemcpyDeviceToDevice, sm));
    // state that must start at zero: the previous call left its own in place
    const float denom = (float)(int)((long long)Nx * Ny * Nz);
    noalloc_reset_kernel<<<1, 1, 0, sm>>>(ctl, maxIt, errBound, denom);
    NA_TRY(cudaGetLastError());
    for (int k = 0; k < 3; ++k)
        NA_TRY(cudaMemsetAsync(b[0][k], 0, (size_t)cells * 4, sm));
    if (maxIt > 0)
        NA_TRY(cudaMemsetAsync(cvg, 0, (size_t)maxIt * 4, sm));

    InitArgs ia;
    memset(&ia, 0, sizeof ia);
    ia.cs = cs;
    ia.ct = ct;
    ia.alpha = al;
    ia.u = uu[0];
    ia.ps = ps[0];
    ia.pt = pt[0];
    ia.ctl = ctl;
    ia.cells = cells;
    ia.label_stride = cells;
    ia.pitch = (int)pitch;
    ia.nr = Ny;
    ia.nlab = 1;
    ia.alpha_labels = 1;
    const int flags = opt ? opt->flags : 0;
    if (maxIt >= 1 && !(flags & ASETS_FLAG_NO_ALPHA_CHECK)) {
        NA_TRY(launch_validate_alpha(ia, d->num_sms, sm));
        int bad = 0;
        NA_TRY(cudaMemcpyAsync(&bad, &ctl->alpha_bad, sizeof bad, cudaMemcpyDeviceToHost, sm));
        NA_TRY(cudaStreamSynchronize(sm));
        if (bad)
            return na_fail(ASETS_ERR_ALPHA, "alpha(x) must be positive. Exiting...");
    }
    NA_TRY(launch_init(0, ia, d->num_sms, sm));

    // kernel variant and arguments (the same fused kernel as the other entry points)
    const int exact = (flags & ASETS_FLAG_EXACT) ? 1 : 0;
    int nv = 0;
    const StencilVariant *tab = stencil_variants(3, EPI_BINARY, exact, &nv);
    const StencilVariant *v = nv > 0 ? &tab[0] : nullptr;
    if (!v)
        return na_fail(ASETS_ERR_UNSUPPORTED, "no kernel variant");
    StencilProblem p;
    memset(&p, 0, sizeof p);
    p.nr = Ny;
    p.nc = Nx;
    p.ns = Nz;
    p.pitch = pitch;
    p.plane = pitch * Nx;
    p.cells = cells;
    p.flow_labels = 1;
    for (int par = 0; par < 2; ++par) {
        for (int k = 0; k < 3; ++k)
            p.b[par][k] = b[par][k];
        p.src[par][0] = ps[par];
        p.src[par][1] = pt[par];
        p.src[par][2] = uu[par];
        p.dst_s[par][0] = ps[par ^ 1];
        p.dst_s[par][1] = pt[par ^ 1];
        p.dst_s[par][2] = uu[par ^ 1];
    }
    p.src_labels[0] = p.src_labels[1] = p.src_labels[2] = 1;
    p.alpha = al;
    p.alpha_labels = 1;
    p.cs = cs;
    p.ct = ct;
    ProblemDesc A;
    const int r = build_problem_desc(reinterpret_cast<EncodeTiledFn>(d->encode), *v, p, &A);
    if (r)
        return na_fail(ASETS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", r);
    NA_TRY(cudaFuncSetAttribute(v->fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                v->smem_bytes));
    int per_sm = 0;
    NA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v->fn, v->nt, v->smem_bytes));
    if (per_sm < 1)
        return na_fail(ASETS_ERR_UNSUPPORTED, "the iteration kernel does not fit on an SM");
    const long long slots = (long long)d->num_sms * per_sm;
    A.zchunks = choose_zchunks(p, *v, slots);
    const int items = problem_items(p, *v, A.zchunks);
    if (items > kMaxItems)
        return na_fail(ASETS_ERR_INVALID_ARG, "problem splits into %d work items; the "
                       "allocation-free entry point handles at most %d", items, kMaxItems);
    A.item_begin = 0;
    A.n_items = items;
    A.ctl = ctl;
    A.item_partials = item_partials;
    A.cvg = cvg;
    A.cc = cc;
    A.inv_cc = 1.0f / cc;
    A.steps = steps;
    NA_TRY(cudaMemcpyAsync(d_desc, &A, sizeof A, cudaMemcpyHostToDevice, sm));
    NA_TRY(cudaMemsetAsync(item_problem, 0, sizeof(int) * items, sm));
    NA_TRY(cudaMemsetAsync(queue, 0, kQueueBytes, sm));
    BatchArgs bargs;
    bargs.probs = d_desc;
    bargs.item_problem = item_problem;
    bargs.total_items = items;
    bargs.queue = queue;
    bargs.done_count = queue + 2;
    long long grid = items;
    if (grid > slots)
        grid = slots;
    if (grid > kMaxBlocks)
        grid = kMaxBlocks;
    if (grid < 1)
        grid = 1;

    // Iterations are queued in chunks; after each chunk the host reads the
    // control block's done flag and stops queueing once erriter has met
    // errBound (a launch queued after that returns at entry).
    void *params[] = {&bargs};
    for (int i0 = 0; i0 < maxIt; i0 += kLaunchChunk) {
        const int i1 = (maxIt - i0 < kLaunchChunk) ? maxIt : i0 + kLaunchChunk;
        for (int i = i0; i < i1; ++i)
            NA_TRY(cudaLaunchKernel(v->fn, dim3((unsigned)grid), dim3(v->nt), params,
                                    v->smem_bytes, sm));
        if (i1 < maxIt) {
            int done = 0;
            NA_TRY(cudaMemcpyAsync(&done, &ctl->done, sizeof done, cudaMemcpyDeviceToHost, sm));
            NA_TRY(cudaStreamSynchronize(sm));
            if (done)
                break;
        }
    }
    IterControl out;
    NA_TRY(cudaMemcpyAsync(&out, ctl, sizeof out, cudaMemcpyDeviceToHost, sm));
    NA_TRY(cudaStreamSynchronize(sm));
    if (out.error & DEV_ERR_TIMEOUT)
        return na_fail(ASETS_ERR_TIMEOUT, "a device-side wait timed out");
    const int final_par = (maxIt == 0) ? 0 : ((out.last_iter + 1) & 1);
    NA_TRY(cudaMemcpy2DAsync(u, (size_t)Ny * 4, uu[final_par], pitch * 4, (size_t)Ny * 4, rows,
                             cudaMemcpyDeviceToDevice, sm));
    NA_TRY(cudaStreamSynchronize(sm));
    *itNum = (maxIt == 0) ? 0 : out.it_num;
    return ASETS_OK;
#undef NA_TRY
}

}  // namespace
