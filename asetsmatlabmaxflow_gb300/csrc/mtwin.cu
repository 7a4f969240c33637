// Matlab-semantics solvers: the GPU form of the reference's Matlab twins of
// the six mex solvers (maxflow/asetsBinaryMF2D.m, asetsBinaryMF3D.m,
// asetsPotts2D.m, asetsPotts3D.m, asetsIshikawa2D.m, asetsIshikawa3D.m),
// the path its tutorials use with gpuArray (tutorials/t03_usingCUDA.m).
// They differ from the mex files: they compute in the class of Ct (single
// or double), break on erriter < beta, initialise Potts/Ishikawa from the
// argmin of Ct, and use Matlab's own expression orders, all kept here;
// the kernels are templated on the element type and follow each .m line's
// evaluation order (IEEE operations, no contraction), so u matches a numpy
// restatement in the same precision bit for bit.
//
// Per iteration, over every flow label (binary 1, Potts L, Ishikawa L-1):
//   1 gradient step of the face flows from ud = divp - ((A - B) + u/cc) of
//     the cell and the one below, (A, B) = (ps, pt) binary, (ps, pt_k)
//     Potts, (pt_k, pt_k+1) Ishikawa
//   2 projection factor gk = 1/max(1, |p|/alpha) per cell
//   3 face flows *= 0.5 (gk + gk of the cell below)
//   4 per cell: divp of every label, then the model's sink/source flows and
//     multipliers, erriter and the next iteration's ud; the last block
//     records erriter and the break.
// Single precision runs 1+2 and 3+4 as two passes (each cell also forms
// the faces above it, which their own cells store); double precision, where
// the FP64 pipe bounds the passes and recomputed faces would cost more
// than the passes, runs the four, and keeps u/cc (the same quotient in 1
// and 4 of an iteration, twice in 4 for Ishikawa) beside u, divided once
// where u is written.
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "asets.h"
#include "internal.h"

using namespace asets;

namespace {

constexpr int kThreads = 256;
enum { MT_BINARY = 0, MT_POTTS = 1, MT_ISHIKAWA = 2 };

struct MTCtl {
    int iter, done, it_num;
    unsigned int ticket;
    int max_it;
    double beta, vol;
};

template <class T>
struct MTArgs {
    int rows, cols, slices, nlab, nflow;
    long long n, f1, f2, f3;  // cells and faces per flow label
    T cc, steps, half, one_over_cc, one_over_ccl, beta;
    const T *cs, *ct, *alpha;
    T *u, *ucc, *ud, *pt, *ps, *divp, *gk, *p1, *p2, *p3, *q1, *q2, *q3;
    double *partials;
    T *erriter;
    MTCtl *ctl;
};

template <class T> __device__ __forceinline__ T add(T a, T b);
template <class T> __device__ __forceinline__ T sub(T a, T b);
template <class T> __device__ __forceinline__ T mul(T a, T b);
template <class T> __device__ __forceinline__ T dvd(T a, T b);
template <class T> __device__ __forceinline__ T sqr(T a);
template <> __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ float dvd(float a, float b) { return __fdiv_rn(a, b); }
template <> __device__ __forceinline__ float sqr(float a) { return __fsqrt_rn(a); }
template <> __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
template <> __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }
template <> __device__ __forceinline__ double sqr(double a) { return __dsqrt_rn(a); }

// u/cc of element o: kept beside u in double precision, divided here in single
template <class T>
__device__ __forceinline__ T u_cc(const MTArgs<T> &A, long long o, T u)
{
    if constexpr (sizeof(T) == 8)
        return A.ucc[o];
    else
        return dvd(u, A.cc);
}
template <class T>
__device__ __forceinline__ T u_cc(const MTArgs<T> &A, long long o)
{
    if constexpr (sizeof(T) == 8)
        return A.ucc[o];
    else
        return dvd(A.u[o], A.cc);
}
// stores u of element o (and, in double precision, u/cc beside it);
// returns the new u/cc
template <class T>
__device__ __forceinline__ T set_u(const MTArgs<T> &A, long long o, T v)
{
    A.u[o] = v;
    const T q = dvd(v, A.cc);
    if constexpr (sizeof(T) == 8)
        A.ucc[o] = q;
    return q;
}

// Matlab's min(a, b) for ordered values; a NaN a is kept (as the restatement)
template <class T>
__device__ __forceinline__ T mn(T a, T b)
{
    return (a <= b || a != a) ? a : b;
}

// Cell coordinates in 32-bit unsigned arithmetic: every index of a solve
// (cells and faces times labels) is below 2^31 (entry check), and a 64-bit
// division costs several times a 32-bit one.
template <class T>
struct Cell {
    int y, x, z;
    long long g;
    __device__ Cell(const MTArgs<T> &A, long long g_) : g(g_)
    {
        const unsigned int gg = (unsigned int)g_;
        const unsigned int q = gg / (unsigned int)A.rows;
        y = (int)(gg - q * (unsigned int)A.rows);
        const unsigned int z_ = q / (unsigned int)A.cols;
        x = (int)(q - z_ * (unsigned int)A.cols);
        z = (int)z_;
    }
};

// label of the element t of a label-major loop over n cells per label
__device__ __forceinline__ int label_of(long long t, long long n)
{
    return (int)((unsigned int)t / (unsigned int)n);
}
// face arrays: p1 rows x (cols+1) x slices (along columns), p2 (rows+1) x
// cols x slices (along rows), p3 rows x cols x (slices+1) (along slices)
template <class T>
__device__ __forceinline__ long long j1(const MTArgs<T> &A, int y, int x, int z)
{
    return ((long long)z * (A.cols + 1) + x) * A.rows + y;
}
template <class T>
__device__ __forceinline__ long long j2(const MTArgs<T> &A, int y, int x, int z)
{
    return ((long long)z * A.cols + x) * (A.rows + 1) + y;
}
template <class T>
__device__ __forceinline__ long long j3(const MTArgs<T> &A, int y, int x, int z)
{
    return ((long long)z * A.cols + x) * A.rows + y;
}

template <class T>
__device__ __forceinline__ bool finished(const MTArgs<T> &A)
{
    return *(volatile int *)&A.ctl->done != 0;
}

#define MT_LOOP(total)                                                                 \
    for (long long t = blockIdx.x * (long long)kThreads + threadIdx.x; t < (total);    \
         t += (long long)gridDim.x * kThreads)

// ud of flow label k at cell g: divp - ((A - B) + u/cc)
template <class T, int M>
__device__ __forceinline__ T ud(const MTArgs<T> &A, int k, long long g)
{
    const long long o = (long long)k * A.n + g;
    T a, b;
    if (M == MT_BINARY) {
        a = A.ps[g];
        b = A.pt[g];
    } else if (M == MT_POTTS) {
        a = A.ps[g];
        b = A.pt[o];
    } else {
        a = A.pt[o];
        b = A.pt[o + A.n];
    }
    return sub(A.divp[o], add(sub(a, b), u_cc(A, o)));
}

// ud of every flow label and cell of the initial state; the cell pass forms
// it for the next iteration
template <class T, int M>
__global__ void mt_ud(const MTArgs<T> A)
{
    MT_LOOP(A.n * A.nflow)
    {
        const int k = label_of(t, A.n);
        A.ud[t] = ud<T, M>(A, k, t - (long long)k * A.n);
    }
}

// gradient step of a face flow pp from the ud of the face's upper and lower
// cells: binary pp + steps*(d); Potts/Ishikawa steps*(d) + pp
template <class T, int M>
__device__ __forceinline__ T face_step(const MTArgs<T> &A, T pp, T ud_up, T ud_lo)
{
    const T s = mul(A.steps, sub(ud_up, ud_lo));
    return (M == MT_BINARY) ? add(pp, s) : add(s, pp);
}

// projection rescale of a face flow: 0.5 (gk of the upper cell + gk of the lower) p
template <class T>
__device__ __forceinline__ T face_rescale(const MTArgs<T> &A, T p, T g_up, T g_lo)
{
    return mul(mul(A.half, add(g_up, g_lo)), p);
}

// projection factor 1/max(1, |p|/alpha) from the sum of squares s of the
// cell's faces; 1/1 is exactly 1, so no division below alpha
template <class T>
__device__ __forceinline__ T proj_factor(const MTArgs<T> &A, T s, T al)
{
    const T g = sqr(mul(s, A.half));
    return (g <= al) ? (T)1 : dvd((T)1, dvd(g, al));
}

// ---- double precision: four passes, each face formed once --------------

template <class T, int M, int D>
__global__ void mt_step(const MTArgs<T> A)
{
    if (finished(A))
        return;
    MT_LOOP(A.n * A.nflow)
    {
        const int k = label_of(t, A.n);
        const Cell<T> c(A, t - (long long)k * A.n);
        const T u0 = A.ud[t];
        auto upd = [&](T *f, T nb) { *f = face_step<T, M>(A, *f, u0, nb); };
        if (c.x >= 1)
            upd(A.p1 + (long long)k * A.f1 + j1(A, c.y, c.x, c.z), A.ud[t - A.rows]);
        if (c.y >= 1)
            upd(A.p2 + (long long)k * A.f2 + j2(A, c.y, c.x, c.z), A.ud[t - 1]);
        if (D == 3 && c.z >= 1)
            upd(A.p3 + (long long)k * A.f3 + j3(A, c.y, c.x, c.z),
                A.ud[t - (long long)A.rows * A.cols]);
    }
}

template <class T, int M, int D>
__global__ void mt_gk(const MTArgs<T> A)
{
    if (finished(A))
        return;
    MT_LOOP(A.n * A.nflow)
    {
        const int k = label_of(t, A.n);
        const Cell<T> c(A, t - (long long)k * A.n);
        const T *f1 = A.p1 + (long long)k * A.f1, *f2 = A.p2 + (long long)k * A.f2;
        const T a = f1[j1(A, c.y, c.x, c.z)], b = f1[j1(A, c.y, c.x + 1, c.z)];
        const T d = f2[j2(A, c.y, c.x, c.z)], e = f2[j2(A, c.y + 1, c.x, c.z)];
        T s = add(mul(a, a), mul(b, b));
        s = add(s, mul(d, d));
        s = add(s, mul(e, e));
        if (D == 3) {
            const T *f3 = A.p3 + (long long)k * A.f3;
            const T p = f3[j3(A, c.y, c.x, c.z)], q = f3[j3(A, c.y, c.x, c.z + 1)];
            s = add(s, mul(p, p));
            s = add(s, mul(q, q));
        }
        A.gk[t] = proj_factor(A, s, A.alpha[t]);
    }
}

template <class T, int M, int D>
__global__ void mt_rescale(const MTArgs<T> A)
{
    if (finished(A))
        return;
    MT_LOOP(A.n * A.nflow)
    {
        const int k = label_of(t, A.n);
        const Cell<T> c(A, t - (long long)k * A.n);
        const T g0 = A.gk[t];
        auto sc = [&](T *f, T gnb) { *f = face_rescale(A, *f, g0, gnb); };
        if (c.x >= 1)
            sc(A.p1 + (long long)k * A.f1 + j1(A, c.y, c.x, c.z), A.gk[t - A.rows]);
        if (c.y >= 1)
            sc(A.p2 + (long long)k * A.f2 + j2(A, c.y, c.x, c.z), A.gk[t - 1]);
        if (D == 3 && c.z >= 1)
            sc(A.p3 + (long long)k * A.f3 + j3(A, c.y, c.x, c.z), A.gk[t - (long long)A.rows * A.cols]);
    }
}

template <class T, int D>
__device__ __forceinline__ T divergence(const MTArgs<T> &A, int k, const Cell<T> &c)
{
    const T *f1 = A.p1 + (long long)k * A.f1, *f2 = A.p2 + (long long)k * A.f2;
    T d = sub(f1[j1(A, c.y, c.x + 1, c.z)], f1[j1(A, c.y, c.x, c.z)]);
    d = add(d, f2[j2(A, c.y + 1, c.x, c.z)]);
    d = sub(d, f2[j2(A, c.y, c.x, c.z)]);
    if (D == 3) {
        const T *f3 = A.p3 + (long long)k * A.f3;
        d = add(d, f3[j3(A, c.y, c.x, c.z + 1)]);
        d = sub(d, f3[j3(A, c.y, c.x, c.z)]);
    }
    return d;
}

// ---- single precision: two passes ---------------------------------------
// The gradient step and the projection factor in one pass, the rescale and
// the cell update in the other.  A cell steps (rescales) its lower faces and
// stores them, and forms its upper faces, which the cells above store, from
// the same operands for its magnitude (divergence).  The stepped flows go
// to the second face buffer (q), the rescaled ones back to p, so that no
// pass reads a face another thread of it writes.

// A cell's value of a per-cell array with those of its lower and upper
// neighbours along each axis, and the cell's lower and upper faces of the
// three face arrays, all loaded before any is used (the passes are bound
// by the latency of these loads).  A neighbour outside the volume reads
// the cell itself; its value is not used.
template <class T, int D>
struct Around {
    T v, xl, xu, yl, yu, zl, zu;  // per-cell values
    T a, b, d, e, p, q;           // faces: x lower/upper, y lower/upper, z lower/upper
    long long fa, fd, fp;         // the lower faces' indices
    bool has_xl, has_xu, has_yl, has_yu, has_zl, has_zu;
    __device__ __forceinline__ Around(const MTArgs<T> &A, const Cell<T> &c, const T *cell,
                                      const T *f1, const T *f2, const T *f3)
    {
        const long long g = c.g, pl = (long long)A.rows * A.cols;
        has_xl = c.x >= 1;
        has_xu = c.x + 1 < A.cols;
        has_yl = c.y >= 1;
        has_yu = c.y + 1 < A.rows;
        has_zl = D == 3 && c.z >= 1;
        has_zu = D == 3 && c.z + 1 < A.slices;
        fa = j1(A, c.y, c.x, c.z);
        fd = j2(A, c.y, c.x, c.z);
        fp = j3(A, c.y, c.x, c.z);
        v = cell[g];
        xl = cell[has_xl ? g - A.rows : g];
        xu = cell[has_xu ? g + A.rows : g];
        yl = cell[has_yl ? g - 1 : g];
        yu = cell[has_yu ? g + 1 : g];
        a = f1[fa];
        b = f1[j1(A, c.y, c.x + 1, c.z)];
        d = f2[fd];
        e = f2[j2(A, c.y + 1, c.x, c.z)];
        if (D == 3) {
            zl = cell[has_zl ? g - pl : g];
            zu = cell[has_zu ? g + pl : g];
            p = f3[fp];
            q = f3[j3(A, c.y, c.x, c.z + 1)];
        } else {
            zl = zu = p = q = (T)0;  // no slices: unused
        }
    }
};

template <class T, int M, int D>
__global__ void mt_step_gk(const MTArgs<T> A)
{
    if (finished(A))
        return;
    MT_LOOP(A.n * A.nflow)
    {
        const int k = label_of(t, A.n);
        const Cell<T> c(A, t - (long long)k * A.n);
        const Around<T, D> s(A, c, A.ud + (long long)k * A.n, A.p1 + (long long)k * A.f1,
                             A.p2 + (long long)k * A.f2, A.p3 + (long long)k * A.f3);
        const T al = A.alpha[t];
        T *d1 = A.q1 + (long long)k * A.f1, *d2 = A.q2 + (long long)k * A.f2;
        T a = s.a, b = s.b, d = s.d, e = s.e;
        if (s.has_xl) {
            a = face_step<T, M>(A, a, s.v, s.xl);
            d1[s.fa] = a;
        }
        if (s.has_xu)
            b = face_step<T, M>(A, b, s.xu, s.v);
        if (s.has_yl) {
            d = face_step<T, M>(A, d, s.v, s.yl);
            d2[s.fd] = d;
        }
        if (s.has_yu)
            e = face_step<T, M>(A, e, s.yu, s.v);
        T m = add(mul(a, a), mul(b, b));
        m = add(m, mul(d, d));
        m = add(m, mul(e, e));
        if (D == 3) {
            T p = s.p, q = s.q;
            if (s.has_zl) {
                p = face_step<T, M>(A, p, s.v, s.zl);
                A.q3[(long long)k * A.f3 + s.fp] = p;
            }
            if (s.has_zu)
                q = face_step<T, M>(A, q, s.zu, s.v);
            m = add(m, mul(p, p));
            m = add(m, mul(q, q));
        }
        A.gk[t] = proj_factor(A, m, al);
    }
}

// divergence of flow label k at cell c from the stepped flows (q), with the
// rescale of every face; the cell's lower faces are stored (into p)
template <class T, int D>
__device__ __forceinline__ T rescaled_divergence(const MTArgs<T> &A, int k, const Cell<T> &c)
{
    const Around<T, D> s(A, c, A.gk + (long long)k * A.n, A.q1 + (long long)k * A.f1,
                         A.q2 + (long long)k * A.f2, A.q3 + (long long)k * A.f3);
    T a = s.a, b = s.b, d = s.d, e = s.e;
    if (s.has_xl) {
        a = face_rescale(A, a, s.v, s.xl);
        A.p1[(long long)k * A.f1 + s.fa] = a;
    }
    if (s.has_xu)
        b = face_rescale(A, b, s.xu, s.v);
    if (s.has_yl) {
        d = face_rescale(A, d, s.v, s.yl);
        A.p2[(long long)k * A.f2 + s.fd] = d;
    }
    if (s.has_yu)
        e = face_rescale(A, e, s.yu, s.v);
    T dv = sub(b, a);
    dv = add(dv, e);
    dv = sub(dv, d);
    if (D == 3) {
        T p = s.p, q = s.q;
        if (s.has_zl) {
            p = face_rescale(A, p, s.v, s.zl);
            A.p3[(long long)k * A.f3 + s.fp] = p;
        }
        if (s.has_zu)
            q = face_rescale(A, q, s.zu, s.v);
        dv = add(dv, q);
        dv = sub(dv, p);
    }
    return dv;
}

// ---- the cell update (both precisions) -----------------------------------

// binary: ps, pt, u of cell g from its divp dv and old u, pt, Cs, Ct, then
// the next iteration's ud; returns |erru|
template <class T>
__device__ __forceinline__ double binary_update(const MTArgs<T> &A, long long g, T dv, T u, T pt0,
                                                T cs, T ct)
{
    const T uc = u_cc(A, g, u);
    const T ps = mn(add(sub(add(dv, pt0), uc), A.one_over_cc), cs);
    const T pt = mn(add(add(-dv, ps), uc), ct);
    const T e = mul(A.cc, sub(add(dv, pt), ps));
    A.ps[g] = ps;
    A.pt[g] = pt;
    const T q = set_u(A, g, sub(u, e));
    A.ud[g] = sub(dv, add(sub(ps, pt), q));
    return fabs((double)e);
}

// The model's sink/source flows and multipliers of cell g from divp of
// every flow label, then the ud of the next iteration; returns the cell's
// share of erriter.
template <class T, int M>
__device__ __forceinline__ double cell_update(const MTArgs<T> &A, long long g)
{
    const long long n = A.n;
    double err = 0.0;
    if (M == MT_BINARY) {
        err += binary_update(A, g, A.divp[g], A.u[g], A.pt[g], A.cs[g], A.ct[g]);
    } else if (M == MT_POTTS) {
        const T ps = A.ps[g];
        T pd = (T)0;
        for (int k = 0; k < A.nlab; ++k) {
            const long long o = (long long)k * n + g;
            const T dv = A.divp[o], uc = u_cc(A, o);
            const T pt = mn(add(add(-dv, ps), uc), A.ct[o]);
            A.pt[o] = pt;
            pd = add(pd, sub(add(dv, pt), uc));
        }
        const T psn = add(dvd(pd, (T)A.nlab), A.one_over_ccl);
        A.ps[g] = psn;
        for (int k = 0; k < A.nlab; ++k) {
            const long long o = (long long)k * n + g;
            const T dv = A.divp[o], pt = A.pt[o];
            const T e = mul(A.cc, sub(add(dv, pt), psn));
            const T q = set_u(A, o, sub(A.u[o], e));
            A.ud[o] = sub(dv, add(sub(psn, pt), q));
            err += fabs((double)e);
        }
    } else {
        const int L = A.nlab;
        for (int k = 0; k < L; ++k) {
            const long long o = (long long)k * n + g;
            T v;
            if (k == 0) {
                v = add(sub(add(A.divp[g], A.pt[g + n]), u_cc(A, g)), A.one_over_cc);
            } else {
                const long long ob = o - n;  // label k-1: its pt is the new one
                v = add(add(-A.divp[ob], A.pt[ob]), u_cc(A, ob));
                if (k < L - 1) {
                    v = sub(add(add(v, A.divp[o]), A.pt[o + n]), u_cc(A, o));
                    v = dvd(v, (T)2);
                }
            }
            A.pt[o] = mn(v, A.ct[o]);
        }
        for (int k = 0; k < L - 1; ++k) {
            const long long o = (long long)k * n + g;
            const T dv = A.divp[o], pa = A.pt[o], pb = A.pt[o + n];
            const T e = mul(A.cc, sub(add(dv, pb), pa));
            const T q = set_u(A, o, sub(A.u[o], e));
            A.ud[o] = sub(dv, add(sub(pa, pb), q));
            err += fabs((double)e);
        }
    }
    return err;
}

// Per cell: divp of every flow label (FUSED: with the rescale of the
// stepped flows), the cell update; the last block records erriter and the
// break.
template <class T, int M, int D, bool FUSED>
__global__ void mt_cell(const MTArgs<T> A)
{
    __shared__ double s_red[kThreads / 32];
    __shared__ int s_last;
    if (finished(A))
        return;
    const int it = *(volatile int *)&A.ctl->iter;
    double err = 0.0;
    MT_LOOP(A.n)
    {
        const Cell<T> c(A, t);
        if (M == MT_BINARY && FUSED) {
            // the cell's own operands are loaded with the divergence's; divp
            // is used by this thread alone and not stored
            const T u = A.u[t], pt = A.pt[t], cs = A.cs[t], ct = A.ct[t];
            const T dv = rescaled_divergence<T, D>(A, 0, c);
            err += binary_update(A, t, dv, u, pt, cs, ct);
            continue;
        }
        for (int k = 0; k < A.nflow; ++k)
            A.divp[(long long)k * A.n + t] =
                FUSED ? rescaled_divergence<T, D>(A, k, c) : divergence<T, D>(A, k, c);
        err += cell_update<T, M>(A, t);
    }
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
        const T e = (T)(tot / A.ctl->vol);
        A.erriter[it] = e;
        if (e < A.beta) {
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

// initial state (the .m files before their loop)
template <class T, int M>
__global__ void mt_init(const MTArgs<T> A)
{
    MT_LOOP(A.n)
    {
        const long long g = t, n = A.n;
        if (M == MT_BINARY) {
            const T cs = A.cs[g], ct = A.ct[g];
            set_u(A, g, (sub(cs, ct) >= (T)0) ? (T)1 : (T)0);
            const T ps = mn(cs, ct);
            A.ps[g] = ps;
            A.pt[g] = ps;
            continue;
        }
        // [m, I] = min(Ct, [], labels): the first minimum
        T m = A.ct[g];
        int I = 0;
        for (int k = 1; k < A.nlab; ++k) {
            const T v = A.ct[(long long)k * n + g];
            if (v < m) {
                m = v;
                I = k;
            }
        }
        for (int k = 0; k < A.nlab; ++k)
            A.pt[(long long)k * n + g] = m;
        if (M == MT_POTTS) {
            A.ps[g] = m;
            for (int k = 0; k < A.nlab; ++k)
                set_u(A, (long long)k * n + g, (I == k) ? (T)1 : (T)0);
        } else {
            for (int k = 0; k < A.nlab - 1; ++k)  // u(:,:,k) = init > k, 1-based
                set_u(A, (long long)k * n + g, (I > k) ? (T)1 : (T)0);
        }
    }
}

int mt_grid(long long n, int sms)
{
    long long b = (n + kThreads - 1) / kThreads;
    const long long cap = (long long)sms * 8;
    return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

template <class T, int M, int D>
asets_status mt_run(asets_context *ctx, int rows, int cols, int slices, int nlab,
                    const void *Cs, const void *Ct, const void *alpha, int iterNum, double beta,
                    double cc, double steps, void *u_out, void *err_out, int *itNum)
{
    cudaStream_t st = context_stream(ctx);
    const int sms = context_num_sms(ctx);
    MTArgs<T> A;
    memset(&A, 0, sizeof A);
    A.rows = rows;
    A.cols = cols;
    A.slices = slices;
    A.nlab = (M == MT_BINARY) ? 1 : nlab;
    A.nflow = (M == MT_ISHIKAWA) ? nlab - 1 : A.nlab;
    const long long n = (long long)rows * cols * slices;
    A.n = n;
    A.f1 = (long long)rows * (cols + 1) * slices;
    A.f2 = (long long)(rows + 1) * cols * slices;
    A.f3 = D == 3 ? (long long)rows * cols * (slices + 1) : 0;
    // scalars rounded to the class of Ct, as Matlab combines them
    A.cc = (T)cc;
    A.steps = (T)steps;
    A.half = (T)0.5;
    A.one_over_cc = (T)(1.0 / cc);
    A.one_over_ccl = (T)(1.0 / (cc * A.nlab));
    A.beta = (T)beta;
    const int nct = A.nlab, nu = (M == MT_ISHIKAWA) ? nlab - 1 : A.nlab;
    const int npt = A.nlab;
    std::vector<void *> bufs;
    auto get = [&](T **p, long long count) {
        void *v = nullptr;
        if (cudaMallocAsync(&v, (size_t)(count < 1 ? 1 : count) * sizeof(T), st) != cudaSuccess)
            return false;
        bufs.push_back(v);
        *p = static_cast<T *>(v);
        return true;
    };
    T *cs = nullptr, *ct = nullptr, *al = nullptr;
    asets_status status = ASETS_OK;
    const int grid = mt_grid(n * A.nflow, sms), gcell = mt_grid(n, sms);
    constexpr bool kFused = sizeof(T) == 4;
    bool ok = get(&ct, n * nct) && get(&al, n * A.nflow) && get(&A.u, n * nu) &&
              get(&A.ud, n * A.nflow) &&
              (!kFused || (get(&A.q1, A.f1 * A.nflow) && get(&A.q2, A.f2 * A.nflow) &&
                           get(&A.q3, A.f3 * A.nflow))) &&
              (sizeof(T) != 8 || get(&A.ucc, n * nu)) && get(&A.pt, n * npt) && get(&A.ps, n) && get(&A.divp, n * A.nflow) &&
              get(&A.gk, n * A.nflow) && get(&A.p1, A.f1 * A.nflow) && get(&A.p2, A.f2 * A.nflow) &&
              get(&A.p3, A.f3 * A.nflow) && get(&A.erriter, iterNum) &&
              (M != MT_BINARY || get(&cs, n));
    void *pv = nullptr;
    ok = ok && cudaMallocAsync(&pv, sizeof(MTCtl) + (size_t)gcell * sizeof(double), st) == cudaSuccess;
    if (ok) {
        bufs.push_back(pv);
        A.ctl = static_cast<MTCtl *>(pv);
        A.partials = reinterpret_cast<double *>(static_cast<char *>(pv) + sizeof(MTCtl));
    }
    cudaError_t e = cudaSuccess;
    MTCtl c0;
    memset(&c0, 0, sizeof c0);
    c0.max_it = iterNum;
    c0.beta = beta;
    c0.vol = (M == MT_BINARY)    ? (double)n
             : (M == MT_POTTS)   ? (double)(n * nlab)
                                 : (double)(n * nlab - 1);  // rows*cols*nlab-1, as the .m files
    if (!ok) {
        status = ASETS_ERR_OUT_OF_MEMORY;
        set_last_error("Matlab-semantics solver: out of device memory");
    } else {
        e = cudaMemcpyAsync(ct, Ct, sizeof(T) * n * nct, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(al, alpha, sizeof(T) * n * A.nflow, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess && M == MT_BINARY)
            e = cudaMemcpyAsync(cs, Cs, sizeof(T) * n, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(A.ctl, &c0, sizeof c0, cudaMemcpyHostToDevice, st);
        // the flows and the second face buffer start at zero; their border
        // faces are never written and stay zero (the zero-flux border)
        T *zero[] = {A.divp, A.p1, A.p2, A.p3, A.erriter, A.q1, A.q2, A.q3};
        const long long fq = kFused ? A.nflow : 0;
        const long long zn[] = {n * A.nflow, A.f1 * A.nflow, A.f2 * A.nflow, A.f3 * A.nflow,
                                (long long)iterNum, A.f1 * fq, A.f2 * fq, A.f3 * fq};
        for (int i = 0; i < 8 && e == cudaSuccess; ++i)
            if (zn[i] > 0)
                e = cudaMemsetAsync(zero[i], 0, sizeof(T) * zn[i], st);
        A.cs = cs;
        A.ct = ct;
        A.alpha = al;
        if (e == cudaSuccess) {
            mt_init<T, M><<<gcell, kThreads, 0, st>>>(A);
            mt_ud<T, M><<<grid, kThreads, 0, st>>>(A);
            e = cudaGetLastError();
        }
        constexpr int kChunk = 16;
        int h_done = 0;
        for (int done_it = 0; e == cudaSuccess && done_it < iterNum; done_it += kChunk) {
            for (int i = 0; i < kChunk && done_it + i < iterNum; ++i) {
                if constexpr (kFused) {
                    mt_step_gk<T, M, D><<<grid, kThreads, 0, st>>>(A);
                    mt_cell<T, M, D, true><<<gcell, kThreads, 0, st>>>(A);
                } else {
                    mt_step<T, M, D><<<grid, kThreads, 0, st>>>(A);
                    mt_gk<T, M, D><<<grid, kThreads, 0, st>>>(A);
                    mt_rescale<T, M, D><<<grid, kThreads, 0, st>>>(A);
                    mt_cell<T, M, D, false><<<gcell, kThreads, 0, st>>>(A);
                }
            }
            e = cudaGetLastError();
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(&h_done, &A.ctl->done, sizeof(int), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(st);
            if (h_done)
                break;
        }
        MTCtl out;
        memset(&out, 0, sizeof out);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&out, A.ctl, sizeof out, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(u_out, A.u, sizeof(T) * n * nu, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && err_out)
            e = cudaMemcpyAsync(err_out, A.erriter, sizeof(T) * iterNum, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
        if (e == cudaSuccess && itNum)
            *itNum = out.it_num;
    }
    if (status == ASETS_OK && e != cudaSuccess) {
        cudaGetLastError();
        status = ASETS_ERR_CUDA;
        set_last_error((std::string("Matlab-semantics solver: ") + cudaGetErrorString(e)).c_str());
    }
    for (void *p : bufs)
        cudaFreeAsync(p, st);
    cudaStreamSynchronize(st);
    return status;
}

template <class T>
asets_status mt_dispatch(int model, int dim, asets_context *ctx, int rows, int cols, int slices,
                         int nlab, const void *Cs, const void *Ct, const void *alpha, int iterNum,
                         double beta, double cc, double steps, void *u, void *err, int *itNum)
{
#define MT_CASE(M, D)                                                                       \
    if (model == M && dim == D)                                                             \
        return mt_run<T, M, D>(ctx, rows, cols, slices, nlab, Cs, Ct, alpha, iterNum, beta, \
                               cc, steps, u, err, itNum);
    MT_CASE(MT_BINARY, 2)
    MT_CASE(MT_BINARY, 3)
    MT_CASE(MT_POTTS, 2)
    MT_CASE(MT_POTTS, 3)
    MT_CASE(MT_ISHIKAWA, 2)
    MT_CASE(MT_ISHIKAWA, 3)
#undef MT_CASE
    set_last_error("Matlab-semantics solver: bad model or dimension");
    return ASETS_ERR_INVALID_ARG;
}

}  // namespace

extern "C" ASETS_API asets_status asets_matlab_solve(
    asets_context *ctx, int model, int precision, int dim, int rows, int cols, int slices,
    int nlab, const void *Cs, const void *Ct, const void *alpha, int iterNum, double beta,
    double cc, double steps, void *u, void *erriter, int *itNum, float *seconds)
{
    if (!ctx || !Ct || !alpha || !u || iterNum < 1 || rows < 1 || cols < 1 || slices < 1 ||
        (dim != 2 && dim != 3) || (dim == 2 && slices != 1) || (precision != 4 && precision != 8) ||
        (model == MT_BINARY && !Cs) || (model == MT_POTTS && nlab < 1) ||
        (model == MT_ISHIKAWA && nlab < 2) || model < 0 || model > 2) {
        set_last_error("asets_matlab_solve: bad arguments");
        return ASETS_ERR_INVALID_ARG;
    }
    if ((long long)(rows + 1) * (cols + 1) * (slices + 1) * (nlab > 1 ? nlab : 1) >= (1LL << 31)) {
        set_last_error("asets_matlab_solve: volume x labels must stay below 2^31 elements");
        return ASETS_ERR_INVALID_ARG;
    }
    const auto t0 = std::chrono::steady_clock::now();
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(context_device(ctx));
    const asets_status s =
        precision == 8 ? mt_dispatch<double>(model, dim, ctx, rows, cols, slices, nlab, Cs, Ct,
                                             alpha, iterNum, beta, cc, steps, u, erriter, itNum)
                       : mt_dispatch<float>(model, dim, ctx, rows, cols, slices, nlab, Cs, Ct,
                                            alpha, iterNum, beta, cc, steps, u, erriter, itNum);
    cudaSetDevice(prev);
    if (seconds)
        *seconds = std::chrono::duration<float>(std::chrono::steady_clock::now() - t0).count();
    return s;
}
