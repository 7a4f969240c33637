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

// mm[0] = key(min), mm[1] = key(max); NaNs are skipped (as Matlab's min/max).
__global__ void minmax_kernel(const float *x, long long n, unsigned int *mm)
{
    unsigned int lo = 0xFFFFFFFFu, hi = 0u;
    for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        const float f = x[i];
        if (f != f)
            continue;
        const unsigned int k = float_key(f);
        lo = min(lo, k);
        hi = max(hi, k);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&mm[0], lo);
        atomicMax(&mm[1], hi);
    }
}

// (I - min) / (max - min), as Matlab's single arithmetic
__device__ __forceinline__ float normalized(float v, const unsigned int *mm)
{
    const float lo = key_float(mm[0]), hi = key_float(mm[1]);
    return __fdiv_rn(__fsub_rn(v, lo), __fsub_rn(hi, lo));
}

__global__ void l1_kernel(const float *img, long long n, Labels m, int L,
                          const unsigned int *mm, float *ct)
{
    for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        const float v = mm ? normalized(img[i], mm) : img[i];
        for (int l = 0; l < L; ++l)
            ct[l * n + i] = fabsf(__fsub_rn(v, m.v[l]));
    }
}

__global__ void neglog_kernel(const float *p, long long total, float eps, float *ct)
{
    for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < total;
         i += (long long)gridDim.x * kThreads)
        ct[i] = -logf(__fadd_rn(p[i], eps));
}

// I' * 255 in single precision as computeLogLikelihoodCost forms it
__device__ __forceinline__ float scaled255(float v, const unsigned int *mm)
{
    return __fmul_rn(normalized(v, mm), 255.0f);
}

// histc(x, 0:255): bin k holds k <= x < k+1, the last bin also x == 255.
__global__ void hist_kernel(const float *img, const int *scrib, long long n, int L,
                            const unsigned int *mm, unsigned int *hist)
{
    __shared__ unsigned int h[kMaxLabels * kBins];
    for (int i = threadIdx.x; i < L * kBins; i += kThreads)
        h[i] = 0;
    __syncthreads();
    for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        const int lab = scrib[i];
        if (lab < 1 || lab > L)
            continue;
        const float x = scaled255(img[i], mm);
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
    for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        const float x = scaled255(img[i], mm);
        int b = (int)roundf(x);
        b = b < 0 ? 0 : (b > kBins - 1 ? kBins - 1 : b);
        for (int l = 0; l < L; ++l)
            ct[l * n + i] = table[l * kBins + b];
    }
}

// alpha = a + b*exp(-c*|grad I'|^p) (p = 1 or 2), replicated over L slices.
__global__ void alpha_kernel(const float *img, int ny, int nx, int nz, const unsigned int *mm,
                             float a, float b, float c, int squared, int L, float *alpha)
{
    const long long n = (long long)ny * nx * nz;
    for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        const int y = (int)(i % ny);
        const long long q = i / ny;
        const int x = (int)(q % nx);
        const int z = (int)(q / nx);
        auto at = [&](int yy, int xx, int zz) {
            const float v = img[((long long)zz * nx + xx) * ny + yy];
            return mm ? normalized(v, mm) : v;
        };
        // Matlab gradient: (f(k+1) - f(k-1))/2 inside, one-sided at the ends
        auto d = [&](int k, int nk, float lo, float mid, float hi) {
            if (nk < 2)
                return 0.f;
            if (k == 0)
                return __fsub_rn(hi, mid);
            if (k == nk - 1)
                return __fsub_rn(mid, lo);
            return __fmul_rn(__fsub_rn(hi, lo), 0.5f);
        };
        const float v = at(y, x, z);
        const float gy = d(y, ny, y > 0 ? at(y - 1, x, z) : v, v, y + 1 < ny ? at(y + 1, x, z) : v);
        const float gx = d(x, nx, x > 0 ? at(y, x - 1, z) : v, v, x + 1 < nx ? at(y, x + 1, z) : v);
        float g2 = __fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy));
        if (nz > 1) {
            const float gz = d(z, nz, z > 0 ? at(y, x, z - 1) : v, v, z + 1 < nz ? at(y, x, z + 1) : v);
            g2 = __fadd_rn(g2, __fmul_rn(gz, gz));
        }
        const float t = squared ? g2 : __fsqrt_rn(g2);
        const float al = __fadd_rn(a, __fmul_rn(b, expf(__fmul_rn(-c, t))));
        for (int l = 0; l < L; ++l)
            alpha[l * n + i] = al;
    }
}

struct Scratch {
    std::vector<void *> ptrs;
    cudaStream_t st;
    explicit Scratch(cudaStream_t s) : st(s) {}
    template <class T>
    cudaError_t get(T **p, size_t bytes)
    {
        void *v = nullptr;
        cudaError_t e = cudaMallocAsync(&v, bytes < 4 ? 4 : bytes, st);
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
    const unsigned int init[2] = {0xFFFFFFFFu, 0u};
    e = cudaMemcpyAsync(*mm, init, sizeof init, cudaMemcpyHostToDevice, s.st);
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
    Scratch s(context_stream(ctx));
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
    Scratch s(context_stream(ctx));
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
    Scratch s(context_stream(ctx));
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
    if (!ctx || !img || !alpha || Ny < 1 || Nx < 1 || Nz < 1 || L < 1) {
        set_last_error("asets_alpha_contrast: bad arguments");
        return ASETS_ERR_INVALID_ARG;
    }
    CtxUse use(ctx);
    const int sms = context_num_sms(ctx);
    const long long n = (long long)Ny * Nx * Nz;
    Scratch s(context_stream(ctx));
    View<float> vi, vo;
    CT_TRY(in_view(s, where, img, (size_t)n, vi));
    CT_TRY(out_view(s, where, alpha, (size_t)n * L, vo));
    unsigned int *mm = nullptr;
    if (normalize)
        CT_TRY(run_minmax(s, vi.d, n, sms, &mm));
    alpha_kernel<<<grid_for(n, sms), kThreads, 0, s.st>>>(vi.d, Ny, Nx, Nz, mm, a, b, c, squared, L,
                                                        vo.d);
    CT_TRY(cudaGetLastError());
    CT_TRY(finish(s, vo));
    CT_TRY(cudaStreamSynchronize(s.st));
    return ASETS_OK;
}
