// Star-shape Potts 2D solver: the continuous max-flow Potts iteration with a
// star-shape prior per label (maxflow/asetsPotts2D_starShape.m, a Matlab
// solver computing in double precision).  The GPU solver computes in FP64
// with every element operation of the .m file in its order, so u matches a
// float64 restatement bit for bit; erriter differs only by summation order.
//
// Per label k, besides the Potts flows (pp1/pp2 spatial flows, pt sink, ps
// source, u multiplier), a multiplier v <= 0 acts along the outward
// direction field ve of the Euclidean distance from the label's seed point,
// and gdv = div(v ve) enters the flow balance (:67-97, :141-170).
//
// One iteration = six passes over all labels (each recomputes the neighbour
// values it needs from the state, so every face is written by one thread;
// u/cc, the same quotient in passes A, D and E of an iteration, is divided
// once, where u is written, and kept beside u; the ud of pass A is formed
// per cell at the end of F and the ud of pass E at the end of D, and the
// gradients read them):
//   A  gradient step of pp1/pp2 from ud = divp + gdv - (ps - pt + u/cc)
//   B  projection factor gk = 1/max(1, |p|/alpha) per cell
//   C  pp1/pp2 *= mean of gk across the face
//   D  divp, pt = min(-(divp + gdv) + ps + u/cc, Ct), ps from the label sum
//   E  v = min(v + stepv * (grad ud . ve), 0)
//   F  gdv = (grad v . ve) + v div ve, u -= cc (divp + gdv + pt - ps), erriter
// The last block of F records erriter and applies the .m file's `<` rule.
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "asets.h"
#include "internal.h"

using namespace asets;

namespace {

constexpr int kThreads = 256;

struct SSCtl {
    int iter, done, it_num;
    unsigned int ticket;
    int max_it;
    double beta, vol;
};

struct SSArgs {
    int rows, cols, nlab;
    long long N;  // rows * cols
    double cc, steps, stepv, inv_ccl;
    const double *ct, *alpha, *ve1, *ve2, *div_ve;
    double *u, *ucc, *ud, *pt, *ps, *divp, *pp1, *pp2, *gk, *v, *gdv;
    double *partials, *erriter;
    SSCtl *ctl;
};

// Flow face arrays: pp1/ve1 are rows x (cols+1), pp2/ve2 (rows+1) x cols.
__device__ __forceinline__ long long f1(const SSArgs &A, int k, int y, int x)
{
    return (long long)k * A.rows * (A.cols + 1) + (long long)x * A.rows + y;
}
__device__ __forceinline__ long long f2(const SSArgs &A, int k, int y, int x)
{
    return (long long)k * (A.rows + 1) * A.cols + (long long)x * (A.rows + 1) + y;
}
__device__ __forceinline__ long long cell(const SSArgs &A, int k, int y, int x)
{
    return (long long)k * A.N + (long long)x * A.rows + y;
}

__device__ __forceinline__ bool finished(const SSArgs &A)
{
    return *(volatile int *)&A.ctl->done != 0;
}

// np.minimum semantics: the first operand when equal or NaN
__device__ __forceinline__ double minimum(double a, double b)
{
    return (a <= b || a != a) ? a : b;
}

// ud of pass A: (divp + gdv) - ((ps - pt) + u/cc)
__device__ __forceinline__ double ud_a(double divp, double gdv, double ps, double pt, double ucc)
{
    return __dsub_rn(__dadd_rn(divp, gdv), __dadd_rn(__dsub_rn(ps, pt), ucc));
}

// ud of pass E: ((gdv + divp) + pt) - (ps + u/cc)
__device__ __forceinline__ double ud_e(double gdv, double divp, double pt, double ps, double ucc)
{
    return __dsub_rn(__dadd_rn(__dadd_rn(gdv, divp), pt), __dadd_rn(ps, ucc));
}

// (label, row, column) of element t of a label-major loop, in 32-bit
// arithmetic (every index is below 2^31: entry check)
struct LabelCell {
    int k, y, x;
    long long g;
    __device__ LabelCell(const SSArgs &A, long long t)
    {
        const unsigned int tt = (unsigned int)t, n = (unsigned int)A.N, r = (unsigned int)A.rows;
        const unsigned int kk = tt / n, gg = tt - kk * n, xx = gg / r;
        k = (int)kk;
        g = gg;
        x = (int)xx;
        y = (int)(gg - xx * r);
    }
};

#define SS_LOOP(total)                                                                 \
    for (long long t = blockIdx.x * (long long)kThreads + threadIdx.x; t < (total);    \
         t += (long long)gridDim.x * kThreads)

__global__ void pass_a(const SSArgs A)
{
    if (finished(A))
        return;
    SS_LOOP(A.N * A.nlab)
    {
        const LabelCell lc(A, t);
        const int k = lc.k, x = lc.x, y = lc.y;
        const double ud = A.ud[t];
        if (x >= 1) {
            const long long f = f1(A, k, y, x);
            A.pp1[f] = __dadd_rn(__dmul_rn(A.steps, __dsub_rn(ud, A.ud[t - A.rows])), A.pp1[f]);
        }
        if (y >= 1) {
            const long long f = f2(A, k, y, x);
            A.pp2[f] = __dadd_rn(__dmul_rn(A.steps, __dsub_rn(ud, A.ud[t - 1])), A.pp2[f]);
        }
    }
}

__global__ void pass_b(const SSArgs A)
{
    if (finished(A))
        return;
    SS_LOOP(A.N * A.nlab)
    {
        const LabelCell lc(A, t);
        const int k = lc.k, x = lc.x, y = lc.y;
        const double a = A.pp1[f1(A, k, y, x)], b = A.pp1[f1(A, k, y, x + 1)];
        const double c = A.pp2[f2(A, k, y, x)], d = A.pp2[f2(A, k, y + 1, x)];
        double s = __dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b));
        s = __dadd_rn(s, __dmul_rn(c, c));
        s = __dadd_rn(s, __dmul_rn(d, d));
        const double n = __dsqrt_rn(__dmul_rn(s, 0.5));
        const double al = A.alpha[t];
        // 1/max(1, n/al); 1/1 is exactly 1, so no division below alpha
        A.gk[t] = (n <= al) ? 1.0 : __ddiv_rn(1.0, __ddiv_rn(n, al));
    }
}

__global__ void pass_c(const SSArgs A)
{
    if (finished(A))
        return;
    SS_LOOP(A.N * A.nlab)
    {
        const LabelCell lc(A, t);
        const int k = lc.k, x = lc.x, y = lc.y;
        const double gc = A.gk[t];
        if (x >= 1) {
            const long long f = f1(A, k, y, x);
            A.pp1[f] = __dmul_rn(__dmul_rn(0.5, __dadd_rn(gc, A.gk[t - A.rows])), A.pp1[f]);
        }
        if (y >= 1) {
            const long long f = f2(A, k, y, x);
            A.pp2[f] = __dmul_rn(__dmul_rn(0.5, __dadd_rn(gc, A.gk[t - 1])), A.pp2[f]);
        }
    }
}

__global__ void pass_d(const SSArgs A)
{
    if (finished(A))
        return;
    SS_LOOP(A.N)
    {
        const unsigned int tt = (unsigned int)t, r = (unsigned int)A.rows;
        const int x = (int)(tt / r), y = (int)(tt - (unsigned int)x * r);
        const double ps = A.ps[t];
        double pd = 0.0;
        for (int k = 0; k < A.nlab; ++k) {
            const long long c = cell(A, k, y, x);
            double dv = __dsub_rn(A.pp1[f1(A, k, y, x + 1)], A.pp1[f1(A, k, y, x)]);
            dv = __dadd_rn(dv, A.pp2[f2(A, k, y + 1, x)]);
            dv = __dsub_rn(dv, A.pp2[f2(A, k, y, x)]);
            A.divp[c] = dv;
            const double s = __dadd_rn(dv, A.gdv[c]);
            const double uc = A.ucc[c];
            const double ud = __dadd_rn(__dadd_rn(-s, ps), uc);
            const double pt = minimum(ud, A.ct[c]);
            A.pt[c] = pt;
            pd = __dadd_rn(pd, __dsub_rn(__dadd_rn(s, pt), uc));
        }
        const double psn = __dadd_rn(__ddiv_rn(pd, (double)A.nlab), A.inv_ccl);
        A.ps[t] = psn;
        // the ud of pass E, from this pass's divp, pt and ps
        for (int k = 0; k < A.nlab; ++k) {
            const long long c = cell(A, k, y, x);
            A.ud[c] = ud_e(A.gdv[c], A.divp[c], A.pt[c], psn, A.ucc[c]);
        }
    }
}

__global__ void pass_e(const SSArgs A)
{
    if (finished(A))
        return;
    SS_LOOP(A.N * A.nlab)
    {
        const LabelCell lc(A, t);
        const int k = lc.k, x = lc.x, y = lc.y;
        const double ud = A.ud[t];
        // vx on the four faces of the cell (border faces stay 0)
        const double vl = x >= 1 ? __dsub_rn(ud, A.ud[t - A.rows]) : 0.0;
        const double vr = x + 1 < A.cols ? __dsub_rn(A.ud[t + A.rows], ud) : 0.0;
        const double vu = y >= 1 ? __dsub_rn(ud, A.ud[t - 1]) : 0.0;
        const double vd = y + 1 < A.rows ? __dsub_rn(A.ud[t + 1], ud) : 0.0;
        double s = __dadd_rn(__dmul_rn(vl, A.ve1[f1(A, k, y, x)]), __dmul_rn(vr, A.ve1[f1(A, k, y, x + 1)]));
        s = __dadd_rn(s, __dmul_rn(vu, A.ve2[f2(A, k, y, x)]));
        s = __dadd_rn(s, __dmul_rn(vd, A.ve2[f2(A, k, y + 1, x)]));
        const double gk = __dmul_rn(s, 0.5);
        const double v = __dadd_rn(A.v[t], __dmul_rn(A.stepv, gk));
        A.v[t] = minimum(v, 0.0);
    }
}

__global__ void pass_f(const SSArgs A)
{
    __shared__ double s_red[kThreads / 32];
    __shared__ int s_last;
    if (finished(A))
        return;
    const int it = *(volatile int *)&A.ctl->iter;
    double err = 0.0;
    SS_LOOP(A.N * A.nlab)
    {
        const LabelCell lc(A, t);
        const int k = lc.k, x = lc.x, y = lc.y;
        const double vc = A.v[t];
        const double vl = x >= 1 ? __dsub_rn(vc, A.v[t - A.rows]) : 0.0;
        const double vr = x + 1 < A.cols ? __dsub_rn(A.v[t + A.rows], vc) : 0.0;
        const double vu = y >= 1 ? __dsub_rn(vc, A.v[t - 1]) : 0.0;
        const double vd = y + 1 < A.rows ? __dsub_rn(A.v[t + 1], vc) : 0.0;
        double s = __dadd_rn(__dmul_rn(vl, A.ve1[f1(A, k, y, x)]), __dmul_rn(vr, A.ve1[f1(A, k, y, x + 1)]));
        s = __dadd_rn(s, __dmul_rn(vu, A.ve2[f2(A, k, y, x)]));
        s = __dadd_rn(s, __dmul_rn(vd, A.ve2[f2(A, k, y + 1, x)]));
        const double gdv = __dadd_rn(__dmul_rn(s, 0.5), __dmul_rn(vc, A.div_ve[t]));
        A.gdv[t] = gdv;
        const double e = __dmul_rn(A.cc, __dsub_rn(__dadd_rn(__dadd_rn(A.divp[t], gdv), A.pt[t]),
                                                  A.ps[lc.g]));
        const double un = __dsub_rn(A.u[t], e);
        const double ucc = __ddiv_rn(un, A.cc);
        A.u[t] = un;
        A.ucc[t] = ucc;
        // the ud of the next iteration's pass A
        A.ud[t] = ud_a(A.divp[t], gdv, A.ps[lc.g], A.pt[t], ucc);
        err += fabs(e);
    }
    // erriter: block partials, the last block sums them in a fixed order
    for (int o = 16; o > 0; o >>= 1)
        err += __shfl_xor_sync(0xffffffffu, err, o);
    if ((threadIdx.x & 31) == 0)
        s_red[threadIdx.x >> 5] = err;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < kThreads / 32; ++w)
            b += s_red[w];
        A.partials[blockIdx.x] = b;
        __threadfence();
        s_last = (atomicAdd(&A.ctl->ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        double tot = 0.0;
        for (unsigned int b = 0; b < gridDim.x; ++b)
            tot += __ldcg(A.partials + b);
        const double e = tot / A.ctl->vol;
        A.erriter[it] = e;
        if (e < A.ctl->beta) {
            A.ctl->done = 1;
            A.ctl->it_num = it + 1;
        } else if (it + 1 >= A.ctl->max_it) {
            A.ctl->done = 1;
            A.ctl->it_num = A.ctl->max_it;
        }
        A.ctl->ticket = 0;
        A.ctl->iter = it + 1;
        __threadfence();
    }
}

// Direction field of the distance from the seed (y0, x0) of label k:
// vd = bwdist in single precision, ve = its forward differences (single,
// stored as double), div_ve in double (:84-97).
__device__ __forceinline__ float seed_dist(int y, int x, int y0, int x0)
{
    const double dy = (double)(y - y0), dx = (double)(x - x0);
    return __double2float_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dx, dx))));
}

__global__ void direction_kernel(const SSArgs A, const int *seeds, double *ve1, double *ve2,
                                 double *div_ve)
{
    SS_LOOP(A.N * A.nlab)
    {
        const LabelCell lc(A, t);
        const int k = lc.k, x = lc.x, y = lc.y;
        const int x0 = seeds[2 * k] - 1, y0 = seeds[2 * k + 1] - 1;
        const float d = seed_dist(y, x, y0, x0);
        // faces at the cell's lower index: interior ones only
        const double e1 = x >= 1 ? (double)__fsub_rn(d, seed_dist(y, x - 1, y0, x0)) : 0.0;
        const double e2 = y >= 1 ? (double)__fsub_rn(d, seed_dist(y - 1, x, y0, x0)) : 0.0;
        ve1[f1(A, k, y, x)] = e1;
        ve2[f2(A, k, y, x)] = e2;
        const double e1r = x + 1 < A.cols ? (double)__fsub_rn(seed_dist(y, x + 1, y0, x0), d) : 0.0;
        const double e2d = y + 1 < A.rows ? (double)__fsub_rn(seed_dist(y + 1, x, y0, x0), d) : 0.0;
        div_ve[t] = __dsub_rn(__dadd_rn(__dsub_rn(e1r, e1), e2d), e2);
        A.ucc[t] = __ddiv_rn(A.u[t], A.cc);  // u/cc of the initial (zero) u
        if (x + 1 == A.cols)
            ve1[f1(A, k, y, x + 1)] = 0.0;
        if (y + 1 == A.rows)
            ve2[f2(A, k, y + 1, x)] = 0.0;
    }
}

__global__ void init_ps_kernel(const SSArgs A)
{
    SS_LOOP(A.N)
    {
        double m = A.ct[t];
        for (int k = 1; k < A.nlab; ++k)
            m = fmin(m, A.ct[(long long)k * A.N + t]);
        A.ps[t] = m;
    }
}

// ud of the first pass A, from the initial state (after init_ps_kernel)
__global__ void init_ud_kernel(const SSArgs A)
{
    SS_LOOP(A.N * A.nlab)
    {
        const LabelCell lc(A, t);
        A.ud[t] = ud_a(A.divp[t], A.gdv[t], A.ps[lc.g], A.pt[t], A.ucc[t]);
    }
}

int ss_grid(long long n, int sms)
{
    long long b = (n + kThreads - 1) / kThreads;
    const long long cap = (long long)sms * 8;
    return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

}  // namespace

extern "C" ASETS_API asets_status asets_potts2d_starshape(
    asets_context *ctx, const double *Ct, const double *alpha, int rows, int cols, int nlab,
    int iterNum, double beta, double cc, double steps, double stepv, const int *init_points,
    double *u, double *erriter, int *itNum, float *seconds)
{
    if (!ctx || !Ct || !alpha || !init_points || !u || !erriter || !itNum || rows < 1 ||
        cols < 1 || nlab < 1 || iterNum < 1) {
        set_last_error("asets_potts2d_starshape: bad arguments");
        return ASETS_ERR_INVALID_ARG;
    }
    const long long N = (long long)rows * cols;
    if (N * nlab >= (1LL << 31)) {
        set_last_error("asets_potts2d_starshape: problem too large");
        return ASETS_ERR_INVALID_ARG;
    }
    for (int k = 0; k < nlab; ++k) {
        const int px = init_points[2 * k], py = init_points[2 * k + 1];
        if (px < 1 || px > cols || py < 1 || py > rows) {
            set_last_error("asets_potts2d_starshape: init point outside the image");
            return ASETS_ERR_INVALID_ARG;
        }
    }
    const auto t0 = std::chrono::steady_clock::now();
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(context_device(ctx));
    cudaStream_t st = context_stream(ctx);
    const int sms = context_num_sms(ctx);
    std::vector<void *> bufs;
    asets_status status = ASETS_OK;
    auto alloc = [&](double **p, long long count) {
        void *v = nullptr;
        if (cudaMallocAsync(&v, (size_t)(count < 1 ? 1 : count) * sizeof(double), st) != cudaSuccess)
            return false;
        bufs.push_back(v);
        *p = static_cast<double *>(v);
        return true;
    };
    SSArgs A;
    memset(&A, 0, sizeof A);
    A.rows = rows;
    A.cols = cols;
    A.nlab = nlab;
    A.N = N;
    A.cc = cc;
    A.steps = steps;
    A.stepv = stepv;
    A.inv_ccl = 1.0 / (cc * (double)nlab);
    const long long NL = N * nlab, F1 = (long long)rows * (cols + 1) * nlab,
                    F2 = (long long)(rows + 1) * cols * nlab;
    double *ct = nullptr, *al = nullptr, *ve1 = nullptr, *ve2 = nullptr, *dve = nullptr;
    const int grid = ss_grid(NL, sms);
    std::vector<double> ct_h(Ct, Ct + NL);
    // hard constraints at the init points (:34-38)
    for (int k = 0; k < nlab; ++k) {
        const long long g = (long long)(init_points[2 * k] - 1) * rows + (init_points[2 * k + 1] - 1);
        for (int l = 0; l < nlab; ++l)
            ct_h[(size_t)(l * N + g)] = 10e11;
        ct_h[(size_t)(k * N + g)] = 0.0;
    }
    int *seeds = nullptr;
    SSCtl c0;
    memset(&c0, 0, sizeof c0);
    c0.max_it = iterNum;
    c0.beta = beta;
    c0.vol = (double)NL;
    int h_done[2] = {0, 0};
    int chunk = 0;
    if (!alloc(&ct, NL) || !alloc(&al, NL) || !alloc(&ve1, F1) || !alloc(&ve2, F2) ||
        !alloc(&dve, NL) || !alloc(&A.u, NL) || !alloc(&A.ucc, NL) || !alloc(&A.ud, NL) || !alloc(&A.pt, NL) || !alloc(&A.ps, N) ||
        !alloc(&A.divp, NL) || !alloc(&A.pp1, F1) || !alloc(&A.pp2, F2) || !alloc(&A.gk, NL) ||
        !alloc(&A.v, NL) || !alloc(&A.gdv, NL) || !alloc(&A.partials, grid) ||
        !alloc(&A.erriter, iterNum)) {
        status = ASETS_ERR_OUT_OF_MEMORY;
        set_last_error("asets_potts2d_starshape: out of device memory");
        goto done;
    }
    {
        void *p = nullptr;
        if (cudaMallocAsync(&p, sizeof(SSCtl) + 2 * nlab * sizeof(int), st) != cudaSuccess) {
            status = ASETS_ERR_OUT_OF_MEMORY;
            goto done;
        }
        bufs.push_back(p);
        A.ctl = static_cast<SSCtl *>(p);
        seeds = reinterpret_cast<int *>(static_cast<char *>(p) + sizeof(SSCtl));
    }
    A.ct = ct;
    A.alpha = al;
    A.ve1 = ve1;
    A.ve2 = ve2;
    A.div_ve = dve;
    {
        cudaError_t e = cudaMemcpyAsync(ct, ct_h.data(), NL * sizeof(double), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(al, alpha, NL * sizeof(double), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(seeds, init_points, 2 * nlab * sizeof(int), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(A.ctl, &c0, sizeof c0, cudaMemcpyHostToDevice, st);
        double *zero[] = {A.u, A.pt, A.divp, A.pp1, A.pp2, A.v, A.gdv, A.erriter};
        const long long zn[] = {NL, NL, NL, F1, F2, NL, NL, iterNum};
        for (int i = 0; i < 8 && e == cudaSuccess; ++i)
            e = cudaMemsetAsync(zero[i], 0, zn[i] * sizeof(double), st);
        if (e == cudaSuccess) {
            direction_kernel<<<grid, kThreads, 0, st>>>(A, seeds, ve1, ve2, dve);
            init_ps_kernel<<<ss_grid(N, sms), kThreads, 0, st>>>(A);
            init_ud_kernel<<<grid, kThreads, 0, st>>>(A);
            e = cudaGetLastError();
        }
        // iterations in chunks; every kernel exits at entry once converged
        constexpr int kChunk = 16;
        for (int done_it = 0; e == cudaSuccess && done_it < iterNum; done_it += kChunk, ++chunk) {
            for (int i = 0; i < kChunk && done_it + i < iterNum; ++i) {
                pass_a<<<grid, kThreads, 0, st>>>(A);
                pass_b<<<grid, kThreads, 0, st>>>(A);
                pass_c<<<grid, kThreads, 0, st>>>(A);
                pass_d<<<ss_grid(N, sms), kThreads, 0, st>>>(A);
                pass_e<<<grid, kThreads, 0, st>>>(A);
                pass_f<<<grid, kThreads, 0, st>>>(A);
            }
            e = cudaGetLastError();
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(&h_done[0], &A.ctl->done, sizeof(int), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(st);
            if (h_done[0])
                break;
        }
        SSCtl out;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&out, A.ctl, sizeof out, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(u, A.u, NL * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(erriter, A.erriter, iterNum * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            cudaGetLastError();
            status = ASETS_ERR_CUDA;
            set_last_error((std::string("asets_potts2d_starshape: ") + cudaGetErrorString(e)).c_str());
        } else {
            *itNum = out.it_num;
        }
    }
done:
    for (void *p : bufs)
        cudaFreeAsync(p, st);
    cudaStreamSynchronize(st);
    cudaSetDevice(prev);
    if (seconds)
        *seconds = std::chrono::duration<float>(std::chrono::steady_clock::now() - t0).count();
    return status;
}
