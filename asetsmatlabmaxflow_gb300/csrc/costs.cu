// Cost terms and regularisation weights built on the GPU: the step before
// the solvers in the reference's applications (applications/*.m), as
// HBM-streaming kernels over the Matlab-layout volume.
//
//   L1 intensity      Ct_l = |I' - m_l|, I' = (I - min I)/(max I - min I)
//                     (L1IntensitySegmentation2D.m:32-45)
//   -log probability  Ct_l = -log(p_l + eps)
//                     (atlasProbabilityMapsRegularization3D.m:39-53)
//   histogram LL      Ct_l = -log10(P_l(bin(I)) + eps) from the 256-bin
//                     histogram of the voxels scribbled with label l
//                     (interactiveGraphCutSegmentation3D.m:47-49, 104-122)
//   contrast alpha    alpha = a + b*exp(-c*|grad I'|^p), central differences
//                     inside, one-sided at the border (Matlab's gradient;
//                     smoothManualSegmentations2D.m:82-91)
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "asets.h"
#include "internal.h"

using namespace asets;

namespace {

constexpr int kThreads = 256;
constexpr int kMaxLabels = 32;
constexpr int kBins = 256;

struct Labels {
    float v[kMaxLabels];
};

int grid_for(long long n, int num_sms)
{
    long long b = (n + kThreads - 1) / kThreads;
    const long long cap = (long long)num_sms * 8;
    return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

// Order-preserving map of floats to unsigned integers (for atomic min/max).
__device__ __forceinline__ unsigned int float_key(float f)
{
    const unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float key_float(unsigned int k)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
#else
    const unsigned int u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

// 16-byte accesses where the arrays allow them (base 16-byte aligned; for
// label-major outputs also n % 4 == 0), so that every thread keeps several
// loads in flight; the remainder element by element.
__device__ __forceinline__ bool aligned16(const void *p)
{
    return (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

// mm[0] = key(min), mm[1] = key(max); NaNs are skipped (as Matlab's min/max).
__global__ void minmax_kernel(const float *x, long long n, unsigned int *mm)
{
    unsigned int lo = 0xFFFFFFFFu, hi = 0u;
    auto take = [&](float f) {
        if (f == f) {
            const unsigned int k = float_key(f);
            lo = min(lo, k);
            hi = max(hi, k);
        }
    };
    const long long t0 = blockIdx.x * (long long)kThreads + threadIdx.x;
    const long long stride = (long long)gridDim.x * kThreads;
    long long head = 0;
    if (aligned16(x)) {
        const long long n4 = n >> 2;
        const float4 *x4 = reinterpret_cast<const float4 *>(x);
#pragma unroll 4
        for (long long i = t0; i < n4; i += stride) {
            const float4 v = __ldg(x4 + i);
            take(v.x);
            take(v.y);
            take(v.z);
            take(v.w);
        }
        head = n4 << 2;
    }
    for (long long i = head + t0; i < n; i += stride)
        take(x[i]);
    // block reduction first: one atomic pair per block (same-address
    // atomics serialise in L2)
    __shared__ unsigned int s_lo[kThreads / 32], s_hi[kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        s_lo[threadIdx.x >> 5] = lo;
        s_hi[threadIdx.x >> 5] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kThreads / 32; ++w) {
            lo = min(lo, s_lo[w]);
            hi = max(hi, s_hi[w]);
        }
        atomicMin(&mm[0], lo);
        atomicMax(&mm[1], hi);
    }
}

// (I - min) / (max - min), as Matlab's single arithmetic; the range is read
// once per thread (mm == nullptr: the identity)
struct Norm {
    float lo = 0.f, den = 1.f;
    bool on = false;
    __device__ explicit Norm(const unsigned int *mm)
    {
        if (mm) {
            lo = key_float(mm[0]);
            den = __fsub_rn(key_float(mm[1]), lo);
            on = true;
        }
    }
    __device__ float operator()(float v) const { return on ? __fdiv_rn(__fsub_rn(v, lo), den) : v; }
};

__global__ void l1_kernel(const float *img, long long n, Labels m, int L,
                          const unsigned int *mm, float *ct)
{
    const Norm nrm(mm);
    const long long t0 = blockIdx.x * (long long)kThreads + threadIdx.x;
    const long long stride = (long long)gridDim.x * kThreads;
    long long head = 0;
    if ((n & 3) == 0 && aligned16(img) && aligned16(ct)) {
        const long long n4 = n >> 2;
        const float4 *x4 = reinterpret_cast<const float4 *>(img);
        float4 *c4 = reinterpret_cast<float4 *>(ct);
#pragma unroll 2
        for (long long i = t0; i < n4; i += stride) {
            const float4 r = __ldg(x4 + i);
            const float v0 = nrm(r.x), v1 = nrm(r.y), v2 = nrm(r.z), v3 = nrm(r.w);
            for (int l = 0; l < L; ++l) {
                const float q = m.v[l];
                __stcs(c4 + l * n4 + i, make_float4(fabsf(__fsub_rn(v0, q)), fabsf(__fsub_rn(v1, q)),
                                                    fabsf(__fsub_rn(v2, q)), fabsf(__fsub_rn(v3, q))));
            }
        }
        head = n;
    }
    for (long long i = head + t0; i < n; i += stride) {
        const float v = nrm(img[i]);
        for (int l = 0; l < L; ++l)
            ct[l * n + i] = fabsf(__fsub_rn(v, m.v[l]));
    }
}

__global__ void neglog_kernel(const float *p, long long total, float eps, float *ct)
{
    auto f = [&](float x) { return -logf(__fadd_rn(x, eps)); };
    const long long t0 = blockIdx.x * (long long)kThreads + threadIdx.x;
    const long long stride = (long long)gridDim.x * kThreads;
    long long head = 0;
    if (aligned16(p) && aligned16(ct)) {
        const long long n4 = total >> 2;
        const float4 *p4 = reinterpret_cast<const float4 *>(p);
        float4 *c4 = reinterpret_cast<float4 *>(ct);
#pragma unroll 2
        for (long long i = t0; i < n4; i += stride) {
            const float4 v = __ldg(p4 + i);
            __stcs(c4 + i, make_float4(f(v.x), f(v.y), f(v.z), f(v.w)));
        }
        head = n4 << 2;
    }
    for (long long i = head + t0; i < total; i += stride)
        ct[i] = f(p[i]);
}

// I' * 255 in single precision as computeLogLikelihoodCost forms it
__device__ __forceinline__ float scaled255(float v, const Norm &nrm)
{
    return __fmul_rn(nrm(v), 255.0f);
}

// histc(x, 0:255): bin k holds k <= x < k+1, the last bin also x == 255.
__global__ void hist_kernel(const float *img, const int *scrib, long long n, int L,
                            const unsigned int *mm, unsigned int *hist)
{
    __shared__ unsigned int h[kMaxLabels * kBins];
    const Norm nrm(mm);
    for (int i = threadIdx.x; i < L * kBins; i += kThreads)
        h[i] = 0;
    __syncthreads();
    for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        const int lab = scrib[i];
        if (lab < 1 || lab > L)
            continue;
        const float x = scaled255(img[i], nrm);
        if (!(x >= 0.f && x <= 255.f))
            continue;
        const int b = min((int)floorf(x), kBins - 1);
        atomicAdd(&h[(lab - 1) * kBins + b], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < L * kBins; i += kThreads)
        if (h[i])
            atomicAdd(&hist[i], h[i]);
}

// Ct_l = cost_l[uint16(I'*255)]: Matlab's uint16() rounds half away from zero.
__global__ void lookup_kernel(const float *img, long long n, int L, const unsigned int *mm,
                              const float *table, float *ct)
{
    const Norm nrm(mm);
    auto bin = [&](float v) {
        const int b = (int)roundf(scaled255(v, nrm));
        return b < 0 ? 0 : (b > kBins - 1 ? kBins - 1 : b);
    };
    const long long t0 = blockIdx.x * (long long)kThreads + threadIdx.x;
    const long long stride = (long long)gridDim.x * kThreads;
    long long head = 0;
    if ((n & 3) == 0 && aligned16(img) && aligned16(ct)) {
        const long long n4 = n >> 2;
        const float4 *x4 = reinterpret_cast<const float4 *>(img);
        float4 *c4 = reinterpret_cast<float4 *>(ct);
        for (long long i = t0; i < n4; i += stride) {
            const float4 v = __ldg(x4 + i);
            const int b0 = bin(v.x), b1 = bin(v.y), b2 = bin(v.z), b3 = bin(v.w);
            for (int l = 0; l < L; ++l) {
                const float *t = table + l * kBins;
                __stcs(c4 + l * n4 + i, make_float4(t[b0], t[b1], t[b2], t[b3]));
            }
        }
        head = n;
    }
    for (long long i = head + t0; i < n; i += stride) {
        const int b = bin(img[i]);
        for (int l = 0; l < L; ++l)
            ct[l * n + i] = table[l * kBins + b];
    }
}

// alpha = a + b*exp(-c*|grad I'|^p) (p = 1 or 2), replicated over L slices.
// A block owns a 32 (rows) x 8 (columns) tile of kAZ planes and walks them
// in order: each thread keeps its column's normalised values of the planes
// z-1, z, z+1 in registers, the tile's plane z and its one-cell halo pass
// through shared memory, so every voxel is read and normalised once (halo
// cells once more).  The raw values are loaded four planes ahead (register
// queues).  At 256^3 the kernel is issue-bound (about 6.5 warp instructions
// per voxel: the IEEE division of the normalisation, expf, the three
// one-sided/central differences), not HBM-bound.
constexpr int kAY = 32, kAX = 8, kAZ = 32;

// Matlab gradient along one axis: (f(k+1) - f(k-1))/2 inside, one-sided at
// the ends, 0 on an axis of length 1
__device__ __forceinline__ float mgrad(int k, int nk, float lo, float mid, float hi)
{
    if (nk < 2)
        return 0.f;
    if (k == 0)
        return __fsub_rn(hi, mid);
    if (k == nk - 1)
        return __fsub_rn(mid, lo);
    return __fmul_rn(__fsub_rn(hi, lo), 0.5f);
}

__global__ void __launch_bounds__(kAY * kAX)
    alpha_kernel(const float *img, int ny, int nx, int nz, const unsigned int *mm, float a,
                 float b, float c, int squared, int L, float *alpha)
{
    __shared__ float pl[kAX + 2][kAY + 2];
    const int ty = threadIdx.x, tx = threadIdx.y;
    const int y = blockIdx.x * kAY + ty, x = blockIdx.y * kAX + tx;
    const int z0 = blockIdx.z * kAZ, z1 = min(nz, z0 + kAZ);
    const bool in = (y < ny && x < nx);
    const long long plane = (long long)ny * nx, n = plane * nz;
    const long long col = (long long)x * ny + y;
    const Norm nrm(mm);
    // halo roles: the first/last row of the tile reads the row outside it,
    // the first/last column the column outside it (inside the volume only)
    const int yy = (ty == 0) ? y - 1 : (ty == kAY - 1 ? y + 1 : -1);
    const int xx = (tx == 0) ? x - 1 : (tx == kAX - 1 ? x + 1 : -1);
    const bool yh = in && yy >= 0 && yy < ny;
    const bool xh = in && xx >= 0 && xx < nx;
    const long long ycol = (long long)x * ny + yy, xcol = (long long)xx * ny + y;
    auto ld = [&](bool ok, int z, long long off) {
        return ok ? __ldg(img + (long long)z * plane + off) : 0.f;
    };
    float v = 0.f, vm = 0.f;
    if (in) {
        v = nrm(img[(long long)z0 * plane + col]);
        vm = z0 > 0 ? nrm(img[(long long)(z0 - 1) * plane + col]) : v;
    }
    // raw centre values of the planes z+1 .. z+4, halo values of z .. z+3
    float c1 = ld(in && z0 + 1 < nz, z0 + 1, col), c2 = ld(in && z0 + 2 < nz, z0 + 2, col);
    float c3 = ld(in && z0 + 3 < nz, z0 + 3, col), c4 = ld(in && z0 + 4 < nz, z0 + 4, col);
    float y0 = ld(yh, z0, ycol), y1 = ld(yh && z0 + 1 < z1, z0 + 1, ycol);
    float y2 = ld(yh && z0 + 2 < z1, z0 + 2, ycol), y3 = ld(yh && z0 + 3 < z1, z0 + 3, ycol);
    float x0 = ld(xh, z0, xcol), x1 = ld(xh && z0 + 1 < z1, z0 + 1, xcol);
    float x2 = ld(xh && z0 + 2 < z1, z0 + 2, xcol), x3 = ld(xh && z0 + 3 < z1, z0 + 3, xcol);
    // unrolled by the queue depth, so that the queues rotate by renaming
    // rather than by moves (a move of a pending load waits for it)
#pragma unroll 4
    for (int z = z0; z < z1; ++z) {
        const float vp = (in && z + 1 < nz) ? nrm(c1) : v;
        const float hyv = yh ? nrm(y0) : v, hxv = xh ? nrm(x0) : v;
        c1 = c2;
        c2 = c3;
        c3 = c4;
        c4 = ld(in && z + 5 < nz, z + 5, col);
        y0 = y1;
        y1 = y2;
        y2 = y3;
        y3 = ld(yh && z + 4 < z1, z + 4, ycol);
        x0 = x1;
        x1 = x2;
        x2 = x3;
        x3 = ld(xh && z + 4 < z1, z + 4, xcol);
        __syncthreads();  // the previous plane's readers are done
        pl[tx + 1][ty + 1] = v;
        // a halo slot is read only by the thread that writes it
        if (in) {
            if (ty == 0)
                pl[tx + 1][0] = hyv;
            if (ty == kAY - 1)
                pl[tx + 1][kAY + 1] = hyv;
            if (tx == 0)
                pl[0][ty + 1] = hxv;
            if (tx == kAX - 1)
                pl[kAX + 1][ty + 1] = hxv;
        }
        __syncthreads();
        if (in) {
            const float gy = mgrad(y, ny, pl[tx + 1][ty], v, pl[tx + 1][ty + 2]);
            const float gx = mgrad(x, nx, pl[tx][ty + 1], v, pl[tx + 2][ty + 1]);
            float g2 = __fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy));
            if (nz > 1) {
                const float gz = mgrad(z, nz, vm, v, vp);
                g2 = __fadd_rn(g2, __fmul_rn(gz, gz));
            }
            const float t = squared ? g2 : __fsqrt_rn(g2);
            const float al = __fadd_rn(a, __fmul_rn(b, expf(__fmul_rn(-c, t))));
            const long long i = (long long)z * plane + col;
            for (int l = 0; l < L; ++l)
                __stcs(alpha + l * n + i, al);
        }
        vm = v;
        v = vp;
    }
}

struct Scratch {
    std::vector<void *> ptrs;
    cudaStream_t st;
    cudaMemPool_t pool;
    explicit Scratch(asets_context *ctx) : st(context_stream(ctx)), pool(context_pool(ctx)) {}
    template <class T>
    cudaError_t get(T **p, size_t bytes)
    {
        void *v = nullptr;
        const size_t b = bytes < 4 ? 4 : bytes;
        cudaError_t e = pool ? cudaMallocFromPoolAsync(&v, b, pool, st) : cudaMallocAsync(&v, b, st);
        if (e == cudaSuccess)
            ptrs.push_back(v);
        *p = static_cast<T *>(v);
        return e;
    }
    ~Scratch()
    {
        for (void *p : ptrs)
            cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
    }
};

#define CT_TRY(call)                                                                       \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            cudaGetLastError();                                                            \
            set_last_error((std::string(#call) + ": " + cudaGetErrorString(e_)).c_str()); \
            return e_ == cudaErrorMemoryAllocation ? ASETS_ERR_OUT_OF_MEMORY : ASETS_ERR_CUDA; \
        }                                                                                  \
    } while (0)

// A device view of a caller array: the array itself, or a device copy of a
// host array (copied back on `finish` for outputs).
template <class T>
struct View {
    T *d = nullptr;
    const T *host_in = nullptr;
    T *host_out = nullptr;
    size_t count = 0;
};

template <class T>
cudaError_t in_view(Scratch &s, asets_memory where, const T *p, size_t count, View<T> &v)
{
    v.count = count;
    if (where == ASETS_DEVICE) {
        v.d = const_cast<T *>(p);
        return cudaSuccess;
    }
    cudaError_t e = s.get(&v.d, count * sizeof(T));
    if (e != cudaSuccess)
        return e;
    return cudaMemcpyAsync(v.d, p, count * sizeof(T), cudaMemcpyHostToDevice, s.st);
}

template <class T>
cudaError_t out_view(Scratch &s, asets_memory where, T *p, size_t count, View<T> &v)
{
    v.count = count;
    if (where == ASETS_DEVICE) {
        v.d = p;
        return cudaSuccess;
    }
    v.host_out = p;
    return s.get(&v.d, count * sizeof(T));
}

template <class T>
cudaError_t finish(Scratch &s, View<T> &v)
{
    if (v.host_out)
        return cudaMemcpyAsync(v.host_out, v.d, v.count * sizeof(T), cudaMemcpyDeviceToHost, s.st);
    return cudaSuccess;
}

cudaError_t run_minmax(Scratch &s, const float *x, long long n, int sms, unsigned int **mm)
{
    cudaError_t e = s.get(mm, 2 * sizeof(unsigned int));
    if (e != cudaSuccess)
        return e;
    // key(min) starts at 0xFFFFFFFF, key(max) at 0 (device-side sets, no
    // staging of a pageable host word)
    e = cudaMemsetAsync(*mm, 0xFF, sizeof(unsigned int), s.st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(*mm + 1, 0, sizeof(unsigned int), s.st);
    if (e != cudaSuccess)
        return e;
    minmax_kernel<<<grid_for(n, sms), kThreads, 0, s.st>>>(x, n, *mm);
    return cudaGetLastError();
}

struct CtxUse {
    int prev = 0;
    explicit CtxUse(asets_context *ctx)
    {
        cudaGetDevice(&prev);
        cudaSetDevice(context_device(ctx));
    }
    ~CtxUse() { cudaSetDevice(prev); }
};

}  // namespace

extern "C" ASETS_API asets_status asets_cost_l1(asets_context *ctx, asets_memory where,
                                                const float *img, long long n,
                                                const float *models, int L, int normalize,
                                                float *Ct)
{
    if (!ctx || !img || !models || !Ct || n < 1 || L < 1 || L > kMaxLabels) {
        set_last_error("asets_cost_l1: bad arguments (1 <= L <= 32)");
        return ASETS_ERR_INVALID_ARG;
    }
    CtxUse use(ctx);
    Scratch s(ctx);
    View<float> vi, vo;
    CT_TRY(in_view(s, where, img, (size_t)n, vi));
    CT_TRY(out_view(s, where, Ct, (size_t)n * L, vo));
    unsigned int *mm = nullptr;
    if (normalize)
        CT_TRY(run_minmax(s, vi.d, n, context_num_sms(ctx), &mm));
    Labels m{};
    for (int l = 0; l < L; ++l)
        m.v[l] = models[l];
    l1_kernel<<<grid_for(n, context_num_sms(ctx)), kThreads, 0, s.st>>>(vi.d, n, m, L, mm, vo.d);
    CT_TRY(cudaGetLastError());
    CT_TRY(finish(s, vo));
    CT_TRY(cudaStreamSynchronize(s.st));
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_cost_neglog(asets_context *ctx, asets_memory where,
                                                    const float *prob, long long n, int L,
                                                    float eps, float *Ct)
{
    if (!ctx || !prob || !Ct || n < 1 || L < 1) {
        set_last_error("asets_cost_neglog: bad arguments");
        return ASETS_ERR_INVALID_ARG;
    }
    CtxUse use(ctx);
    Scratch s(ctx);
    View<float> vi, vo;
    const long long total = n * L;
    CT_TRY(in_view(s, where, prob, (size_t)total, vi));
    CT_TRY(out_view(s, where, Ct, (size_t)total, vo));
    neglog_kernel<<<grid_for(total, context_num_sms(ctx)), kThreads, 0, s.st>>>(vi.d, total, eps,
                                                                               vo.d);
    CT_TRY(cudaGetLastError());
    CT_TRY(finish(s, vo));
    CT_TRY(cudaStreamSynchronize(s.st));
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_cost_histogram_ll(asets_context *ctx, asets_memory where,
                                                          const float *img, const int *scribbles,
                                                          long long n, int L, double eps,
                                                          float *Ct, unsigned int *hist_out)
{
    if (!ctx || !img || !scribbles || !Ct || n < 1 || L < 1 || L > kMaxLabels) {
        set_last_error("asets_cost_histogram_ll: bad arguments (1 <= L <= 32)");
        return ASETS_ERR_INVALID_ARG;
    }
    CtxUse use(ctx);
    const int sms = context_num_sms(ctx);
    Scratch s(ctx);
    View<float> vi, vo;
    View<int> vs;
    CT_TRY(in_view(s, where, img, (size_t)n, vi));
    CT_TRY(in_view(s, where, scribbles, (size_t)n, vs));
    CT_TRY(out_view(s, where, Ct, (size_t)n * L, vo));
    unsigned int *mm = nullptr, *hist = nullptr;
    float *table = nullptr;
    CT_TRY(run_minmax(s, vi.d, n, sms, &mm));
    CT_TRY(s.get(&hist, (size_t)L * kBins * sizeof(unsigned int)));
    CT_TRY(cudaMemsetAsync(hist, 0, (size_t)L * kBins * sizeof(unsigned int), s.st));
    hist_kernel<<<grid_for(n, sms), kThreads, 0, s.st>>>(vi.d, vs.d, n, L, mm, hist);
    CT_TRY(cudaGetLastError());
    // per-bin cost on the host in double, as the reference's binCounts./sum
    // and -log10(P + epsilon)
    std::vector<unsigned int> h((size_t)L * kBins);
    CT_TRY(cudaMemcpyAsync(h.data(), hist, h.size() * sizeof(unsigned int), cudaMemcpyDeviceToHost,
                           s.st));
    CT_TRY(cudaStreamSynchronize(s.st));
    std::vector<float> tab((size_t)L * kBins);
    for (int l = 0; l < L; ++l) {
        double total = 0.0;
        for (int k = 0; k < kBins; ++k)
            total += (double)h[(size_t)l * kBins + k];
        for (int k = 0; k < kBins; ++k) {
            const double p = (double)h[(size_t)l * kBins + k] / total;  // NaN if no scribble
            tab[(size_t)l * kBins + k] = (float)(-std::log10(p + eps));
        }
    }
    if (hist_out)
        memcpy(hist_out, h.data(), h.size() * sizeof(unsigned int));
    CT_TRY(s.get(&table, tab.size() * sizeof(float)));
    CT_TRY(cudaMemcpyAsync(table, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice,
                           s.st));
    lookup_kernel<<<grid_for(n, sms), kThreads, 0, s.st>>>(vi.d, n, L, mm, table, vo.d);
    CT_TRY(cudaGetLastError());
    CT_TRY(finish(s, vo));
    CT_TRY(cudaStreamSynchronize(s.st));
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_alpha_contrast(asets_context *ctx, asets_memory where,
                                                       const float *img, int Ny, int Nx, int Nz,
                                                       int normalize, float a, float b, float c,
                                                       int squared, int L, float *alpha)
{
    if (!ctx || !img || !alpha || Ny < 1 || Nx < 1 || Nz < 1 || L < 1 ||
        (Nx + kAX - 1) / kAX > 65535 || (Nz + kAZ - 1) / kAZ > 65535) {
        set_last_error("asets_alpha_contrast: bad arguments");
        return ASETS_ERR_INVALID_ARG;
    }
    CtxUse use(ctx);
    const int sms = context_num_sms(ctx);
    const long long n = (long long)Ny * Nx * Nz;
    Scratch s(ctx);
    View<float> vi, vo;
    CT_TRY(in_view(s, where, img, (size_t)n, vi));
    CT_TRY(out_view(s, where, alpha, (size_t)n * L, vo));
    unsigned int *mm = nullptr;
    if (normalize)
        CT_TRY(run_minmax(s, vi.d, n, sms, &mm));
    const dim3 agrid((Ny + kAY - 1) / kAY, (Nx + kAX - 1) / kAX, (Nz + kAZ - 1) / kAZ);
    alpha_kernel<<<agrid, dim3(kAY, kAX), 0, s.st>>>(vi.d, Ny, Nx, Nz, mm, a, b, c, squared, L,
                                                      vo.d);
    CT_TRY(cudaGetLastError());
    CT_TRY(finish(s, vo));
    CT_TRY(cudaStreamSynchronize(s.st));
    return ASETS_OK;
}
