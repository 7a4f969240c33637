// Initial state of each model and the alpha(x) > 0 check.
//
//  binary:   u = (Cs - Ct >= 0), ps = pt = min(Cs, Ct)
//            (maxflow/asetsBinaryMF3D_mex.c:205-224)
//  Potts:    ps = min_l Ct, pt_l = ps, u one-hot at the FIRST argmin
//            (asetsPotts3D_mex.c:219-258)
//  Ishikawa: pt_l = min_l Ct for l < L-1 (the top layer stays 0),
//            u_l = (l < argmin) (asetsIshikawa3D_mex.c:230-270)
//
// The argmin search starts from 1e30 / 1e9 and uses `minVal > Ct` exactly
// as the reference, so ties resolve to the lowest label and a pixel whose
// costs are all >= 1e30 (or NaN) keeps the sentinel.
#include "internal.h"
#include "device_common.cuh"

namespace asets {

constexpr int kInitThreads = 256;

__global__ void init_binary_kernel(InitArgs A)
{
    for (long long g = blockIdx.x * (long long)kInitThreads + threadIdx.x; g < A.cells;
         g += (long long)gridDim.x * kInitThreads) {
        if ((int)(g % A.pitch) >= A.nr)
            continue;
        const float cs = A.cs[g], ct = A.ct[g];
        A.u[g] = (cs - ct >= 0.0f) ? 1.0f : 0.0f;
        const float m = min_ref(cs, ct);
        A.ps[g] = m;
        A.pt[g] = m;
    }
}

__device__ __forceinline__ void argmin_labels(const float *ct, long long g, long long S, int L,
                                              float &mv, int &mi)
{
    mv = 1e30f;
    mi = 1000000000;
    for (int l = 0; l < L; ++l) {
        const float v = ct[g + l * S];
        if (mv > v) {
            mv = v;
            mi = l;
        }
    }
}

__global__ void init_potts_kernel(InitArgs A)
{
    const long long S = A.label_stride;
    for (long long g = blockIdx.x * (long long)kInitThreads + threadIdx.x; g < A.cells;
         g += (long long)gridDim.x * kInitThreads) {
        if ((int)(g % A.pitch) >= A.nr)
            continue;
        float mv;
        int mi;
        argmin_labels(A.ct, g, S, A.nlab, mv, mi);
        A.ps[g] = mv;
        for (int l = 0; l < A.nlab; ++l) {
            A.pt[g + l * S] = mv;
            A.u[g + l * S] = (l == mi) ? 1.0f : 0.0f;
        }
    }
}

__global__ void init_ishikawa_kernel(InitArgs A)
{
    const long long S = A.label_stride;
    for (long long g = blockIdx.x * (long long)kInitThreads + threadIdx.x; g < A.cells;
         g += (long long)gridDim.x * kInitThreads) {
        if ((int)(g % A.pitch) >= A.nr)
            continue;
        float mv;
        int mi;
        argmin_labels(A.ct, g, S, A.nlab, mv, mi);
        for (int l = 0; l < A.nlab - 1; ++l) {
            A.pt[g + l * S] = mv;
            A.u[g + l * S] = (l >= mi) ? 0.0f : 1.0f;
        }
        A.pt[g + (A.nlab - 1) * S] = 0.0f;
    }
}

// projStep's check, `if (alpha <= 0) error` (asetsBinaryMF3D_mex.c:317-319),
// over every alpha slice the solve reads.  NaN passes, as in the reference.
__global__ void validate_alpha_kernel(InitArgs A)
{
    int bad = 0;
    const long long total = A.cells * A.alpha_labels;
    for (long long i = blockIdx.x * (long long)kInitThreads + threadIdx.x; i < total;
         i += (long long)gridDim.x * kInitThreads) {
        const long long g = i % A.cells;
        if ((int)(g % A.pitch) >= A.nr)
            continue;
        if (A.alpha[i] <= 0.0f)
            bad = 1;
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0)
        atomicOr(&A.ctl->alpha_bad, 1);
}

static int grid_for(long long n, int num_sms)
{
    long long b = (n + kInitThreads - 1) / kInitThreads;
    long long cap = (long long)num_sms * 8;
    if (b < 1)
        b = 1;
    return (int)(b < cap ? b : cap);
}

cudaError_t launch_init(int model, const InitArgs &a, int num_sms, cudaStream_t st)
{
    const int grid = grid_for(a.cells, num_sms);
    switch (model) {
    case 0: init_binary_kernel<<<grid, kInitThreads, 0, st>>>(a); break;
    case 1: init_potts_kernel<<<grid, kInitThreads, 0, st>>>(a); break;
    case 2: init_ishikawa_kernel<<<grid, kInitThreads, 0, st>>>(a); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_validate_alpha(const InitArgs &a, int num_sms, cudaStream_t st)
{
    validate_alpha_kernel<<<grid_for(a.cells * a.alpha_labels, num_sms), kInitThreads, 0, st>>>(a);
    return cudaGetLastError();
}

// Self-check of the bounded wait: one thread arms an mbarrier for 16 bytes
// of transaction that no copy will deliver and waits on it with the solver
// kernels' bounded wait, which must give up after its budget and report
// DEV_ERR_TIMEOUT.  Nothing is in flight when the kernel returns.
__global__ void wait_selftest_kernel(int *err)
{
    __shared__ uint64_t bar;
    __shared__ int abort_flag;
    if (threadIdx.x == 0) {
        abort_flag = 0;
        mbar_init(&bar, 1);
        mbar_fence_init();
        mbar_arrive_expect_tx(&bar, 16);
        if (!mbar_wait_bounded(&bar, 0, &abort_flag))
            atomicOr(err, DEV_ERR_TIMEOUT);
    }
}

cudaError_t launch_wait_selftest(int *d_err, cudaStream_t st)
{
    wait_selftest_kernel<<<1, 32, 0, st>>>(d_err);
    return cudaGetLastError();
}

}  // namespace asets
