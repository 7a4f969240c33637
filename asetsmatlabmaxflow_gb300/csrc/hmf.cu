// Hierarchical max-flow (HMF), full-flow iteration, 2D and 3D: the GPU form
// of maxflow/asetsHMF2D.m / asetsHMF3D.m (MaxFullFlow), a Matlab class in
// the reference computing in the class of its cost terms (single or double),
// here templated on that type with the .m files' evaluation order.
//
// The label hierarchy is a tree of nodes listed in pre-order (every parent
// before its children, children in their order).  Per iteration:
//   K1 per pixel, all nodes: sink flows children-first (UpdateSinkFlows),
//      then the labels (UpdateLabels), then g = steps*(div + pt - P.pt - u/cc)
//      of every non-root node (the first line of UpdateSpatialFlows) -- all
//      per-pixel, so one pass (with the pixel's nodes staged in shared
//      memory when they fit, k1_staged);
//   K2 gradient step of the spatial flows, K3 flow magnitude and projection
//   factor, K4 flow rescale, K5 divergence (the rest of UpdateSpatialFlows);
//   in 2D without direction fields one tiled kernel runs K2-K5.
// Costs (CalculateCostsFullFlow) are summed on the device in double.
//
// The DAG solver (maxflow/asetsDAGMF2D.m / 3D, nodes may have several
// parents, each child weighted 1/(its number of parents)) shares the spatial
// passes; its iteration is spatial flows first, then one per-pixel pass for
// PushDownFlows (top-down list), PushCapacityUp (bottom-up) and the labels.
//
// Geodesic branch (nodes with direction fields lx, ly (, lz); asetsHMF2D.m
// :228-247, asetsHMF3D.m:215-236, asetsDAGMF2D.m:275-294): the fields are
// normalised once at initialisation (k_norm_dirs); after the gradient step
// k_exempt_a forms per cell the exemption amount a (into g) and
// k_exempt_e per face the exempt flow e, taken off the flow before the
// projection and added back in the rescale.
//
// Pseudo-flow (asetsHMF2D.m / 3D MaxPseudoFlow): one per-pixel pass for the
// capacity reset, push-down, the labels u*exp(-g/cc) normalised over the
// leaves and the push-up of capacity requests, then the same spatial passes
// on steps*g; at the end each inner node's u is the sum of its children's.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "asets.h"
#include "internal.h"

using namespace asets;

namespace {

constexpr int kThreads = 256;

template <class T>
struct NodeDev {
    const T *ct;     // leaves
    const T *alpha;  // per-pixel alpha or null
    T alpha_s;       // scalar alpha
    int parent, child_begin, nchild;
    int nparent;     // DAG: number of parents (parent = the first)
    T wdiv;          // DAG: sum of the children's weights squared (+1 below the root)
    T *l[3];         // direction fields (normalised in place) or null
    int nnorm;       // normalisations at initialisation (DAG: paths from the root)
};

template <class T>
struct HArgs {
    int dim, d1, d2, d3, m;
    int paren;  // gradient step p + (g1 - g0) (asetsHMF2D.m) instead of (p + g1) - g0
    long long n, f1, f2, f3;  // cells and face counts per node
    T cc, steps, inv_cc;      // inv_cc: 1/cc formed in double (the root's 1/cc .* ones)
    const NodeDev<T> *nodes;
    const int *children;
    const T *wchild;    // DAG: weight of each child edge
    const int *order;   // DAG: the top-down node list
    T *pn;              // DAG: pushed-down flow of multi-parent nodes
    T *pt, *u, *div, *g, *p1, *p2, *p3;
    int nedges;         // DAG: child edges (entries of children)
    T *e1, *e2, *e3;  // exempt flow per face (nodes with direction fields)
    double *cost;  // [m][2]: sum u*Ct (leaves), sum u*div (non-root)
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
template <class T> __device__ __forceinline__ T expo(T a);
template <> __device__ __forceinline__ float expo(float a) { return expf(a); }
template <> __device__ __forceinline__ double expo(double a) { return exp(a); }

// pixel c = (z*d2 + x)*d1 + y; face arrays: p1 (d1-1) x d2 x d3, p2
// d1 x (d2-1) x d3, p3 d1 x d2 x (d3-1), each face indexed by the pixel
// before it along its axis.
template <class T>
struct Pix {
    int y, x, z;
    long long c;
    // 32-bit unsigned arithmetic: every index of a solve (pixels times
    // nodes) is below 2^31 (entry check)
    __device__ Pix(const HArgs<T> &A, long long c_) : c(c_)
    {
        const unsigned int cc_ = (unsigned int)c_;
        const unsigned int q = cc_ / (unsigned int)A.d1;
        y = (int)(cc_ - q * (unsigned int)A.d1);
        const unsigned int z_ = q / (unsigned int)A.d2;
        x = (int)(q - z_ * (unsigned int)A.d2);
        z = (int)z_;
    }
};

// node offset of the element t of a node-major loop over n pixels per node
__device__ __forceinline__ int node_of(long long t, long long n)
{
    return (int)((unsigned int)t / (unsigned int)n);
}
template <class T>
__device__ __forceinline__ long long i1(const HArgs<T> &A, int y, int x, int z)
{
    return ((long long)z * A.d2 + x) * (A.d1 - 1) + y;
}
template <class T>
__device__ __forceinline__ long long i2(const HArgs<T> &A, int y, int x, int z)
{
    return ((long long)z * (A.d2 - 1) + x) * A.d1 + y;
}
template <class T>
__device__ __forceinline__ long long i3(const HArgs<T> &A, int y, int x, int z)
{
    return ((long long)z * A.d2 + x) * A.d1 + y;
}

#define H_LOOP(total)                                                                  \
    for (long long t = blockIdx.x * (long long)kThreads + threadIdx.x; t < (total);    \
         t += (long long)gridDim.x * kThreads)

template <class T>
__global__ void k1_pointwise(const HArgs<T> A)
{
    H_LOOP(A.n)
    {
        const long long c = t;
        // sink flows, children before parents (pre-order reversed); a node
        // reads its parent's pt before the parent is updated
        for (int i = A.m - 1; i >= 0; --i) {
            const NodeDev<T> nd = A.nodes[i];
            const long long o = (long long)i * A.n + c;
            T acc;
            if (nd.parent >= 0)
                acc = add(sub(A.pt[(long long)nd.parent * A.n + c], A.div[o]), dvd(A.u[o], A.cc));
            else
                acc = A.inv_cc;
            if (nd.nchild == 0) {
                const T ct = nd.ct[c];
                A.pt[o] = (ct <= acc || ct != ct) ? ct : acc;
                continue;
            }
            for (int j = 0; j < nd.nchild; ++j) {
                const long long oc = (long long)A.children[nd.child_begin + j] * A.n + c;
                acc = sub(add(add(acc, A.pt[oc]), A.div[oc]), dvd(A.u[oc], A.cc));
            }
            A.pt[o] = dvd(acc, (T)(nd.parent >= 0 ? 1 + nd.nchild : nd.nchild));
        }
        // labels, then the flow-gradient input g of every non-root node
        for (int i = 1; i < A.m; ++i) {
            const long long o = (long long)i * A.n + c;
            const T ptp = A.pt[(long long)A.nodes[i].parent * A.n + c];
            const T dv = A.div[o], pt = A.pt[o];
            const T u = add(A.u[o], mul(A.cc, sub(sub(ptp, dv), pt)));
            A.u[o] = u;
            A.g[o] = mul(A.steps, sub(sub(add(dv, pt), ptp), dvd(u, A.cc)));
        }
    }
}

// k1_pointwise with the pixel's values of every node staged in shared
// memory (one column per thread): the pixel's loads are issued together
// and the children-first chain of sink flows runs on shared memory instead
// of reading back through L2 what the thread has just stored.  A leaf's old
// sink flow is never read (its parent reads it after the leaf's update), so
// its slot holds Ct until then.  The node table is staged once per block.
// Same operations in the same order as k1_pointwise.
struct K1Stage {
    // the node table: parent, first child and child count per node and the
    // children list (4m ints), then the nodes' Ct pointers; then the three
    // per-thread columns (sink flow, divergence, label) of every node
    __host__ __device__ static constexpr int ptr_off(int m) { return 16 * m; }
    __host__ __device__ static constexpr int table_bytes(int m) { return 16 * m + (8 * m + 15) / 16 * 16; }
    __host__ __device__ static constexpr int bytes(int m, int elem) { return table_bytes(m) + 3 * m * kThreads * elem; }
};

template <class T>
__global__ void __launch_bounds__(kThreads) k1_staged(const HArgs<T> A)
{
    extern __shared__ __align__(16) unsigned char k1sm[];
    const int m = A.m, tid = threadIdx.x;
    int *npar = reinterpret_cast<int *>(k1sm);
    int *nfirst = npar + m, *ncount = nfirst + m, *kids = ncount + m;
    const T **cts = reinterpret_cast<const T **>(k1sm + K1Stage::ptr_off(m));
    T *PT = reinterpret_cast<T *>(k1sm + K1Stage::table_bytes(m));
    T *DV = PT + m * kThreads, *U = DV + m * kThreads;
    for (int i = tid; i < m; i += kThreads) {
        const NodeDev<T> &nd = A.nodes[i];
        npar[i] = nd.parent;
        nfirst[i] = nd.child_begin;
        ncount[i] = nd.nchild;
        cts[i] = nd.ct;
    }
    for (int j = tid; j < m - 1; j += kThreads)
        kids[j] = A.children[j];
    __syncthreads();
    H_LOOP(A.n)
    {
        const long long c = t;
        for (int i = 0; i < m; ++i) {
            const long long o = (long long)i * A.n + c;
            PT[i * kThreads + tid] = ncount[i] == 0 ? cts[i][c] : A.pt[o];
            if (i > 0) {
                DV[i * kThreads + tid] = A.div[o];
                U[i * kThreads + tid] = A.u[o];
            }
        }
        for (int i = m - 1; i >= 0; --i) {
            const int par = npar[i];
            T acc = par >= 0 ? add(sub(PT[par * kThreads + tid], DV[i * kThreads + tid]),
                                   dvd(U[i * kThreads + tid], A.cc))
                             : A.inv_cc;
            const int nc = ncount[i];
            if (nc == 0) {
                const T ct = PT[i * kThreads + tid];
                PT[i * kThreads + tid] = (ct <= acc || ct != ct) ? ct : acc;
                continue;
            }
            for (int j = 0; j < nc; ++j) {
                const int ch = kids[nfirst[i] + j];
                acc = sub(add(add(acc, PT[ch * kThreads + tid]), DV[ch * kThreads + tid]),
                          dvd(U[ch * kThreads + tid], A.cc));
            }
            PT[i * kThreads + tid] = dvd(acc, (T)(par >= 0 ? 1 + nc : nc));
        }
        A.pt[c] = PT[tid];
        for (int i = 1; i < m; ++i) {
            const long long o = (long long)i * A.n + c;
            const T ptp = PT[npar[i] * kThreads + tid];
            const T dv = DV[i * kThreads + tid], pt = PT[i * kThreads + tid];
            const T u = add(U[i * kThreads + tid], mul(A.cc, sub(sub(ptp, dv), pt)));
            A.pt[o] = pt;
            A.u[o] = u;
            A.g[o] = mul(A.steps, sub(sub(add(dv, pt), ptp), dvd(u, A.cc)));
        }
    }
}

template <class T>
__global__ void k2_gradient(const HArgs<T> A)
{
    H_LOOP(A.n * (A.m - 1))
    {
        const int i = 1 + node_of(t, A.n);
        const Pix<T> p(A, t - (long long)(i - 1) * A.n);
        const T *g = A.g + (long long)i * A.n;
        const T gc = g[p.c];
        // 2D: p + (g(k+1) - g(k)); 3D: (p + g(k+1)) - g(k)
        auto step = [&](T pv, T gn) { return A.paren ? add(pv, sub(gn, gc)) : sub(add(pv, gn), gc); };
        if (p.y + 1 < A.d1) {
            T *f = A.p1 + (long long)i * A.f1 + i1(A, p.y, p.x, p.z);
            *f = step(*f, g[p.c + 1]);
        }
        if (p.x + 1 < A.d2) {
            T *f = A.p2 + (long long)i * A.f2 + i2(A, p.y, p.x, p.z);
            *f = step(*f, g[p.c + A.d1]);
        }
        if (A.dim == 3 && p.z + 1 < A.d3) {
            T *f = A.p3 + (long long)i * A.f3 + i3(A, p.y, p.x, p.z);
            *f = step(*f, g[p.c + (long long)A.d1 * A.d2]);
        }
    }
}

template <class T>
__global__ void k3_projection(const HArgs<T> A)
{
    H_LOOP(A.n * (A.m - 1))
    {
        const int i = 1 + node_of(t, A.n);
        const Pix<T> p(A, t - (long long)(i - 1) * A.n);
        const T *f1 = A.p1 + (long long)i * A.f1;
        const T *f2 = A.p2 + (long long)i * A.f2;
        const T *f3 = A.p3 + (long long)i * A.f3;
        // sum of the squares of the cell's faces, in the .m files' order
        T s = (T)0;
        if (p.y + 1 < A.d1) {
            const T v = f1[i1(A, p.y, p.x, p.z)];
            s = add(s, mul(v, v));
        }
        if (p.y >= 1) {
            const T v = f1[i1(A, p.y - 1, p.x, p.z)];
            s = add(s, mul(v, v));
        }
        if (p.x + 1 < A.d2) {
            const T v = f2[i2(A, p.y, p.x, p.z)];
            s = add(s, mul(v, v));
        }
        if (p.x >= 1) {
            const T v = f2[i2(A, p.y, p.x - 1, p.z)];
            s = add(s, mul(v, v));
        }
        if (A.dim == 3) {
            if (p.z + 1 < A.d3) {
                const T v = f3[i3(A, p.y, p.x, p.z)];
                s = add(s, mul(v, v));
            }
            if (p.z >= 1) {
                const T v = f3[i3(A, p.y, p.x, p.z - 1)];
                s = add(s, mul(v, v));
            }
        }
        const T mag = sqr(s);
        const NodeDev<T> &nd = A.nodes[i];
        const T al = nd.alpha ? nd.alpha[p.c] : nd.alpha_s;
        A.g[(long long)i * A.n + p.c] = (mag <= al) ? (T)1 : dvd(al, mag);
    }
}

template <class T>
__global__ void k4_rescale(const HArgs<T> A)
{
    H_LOOP(A.n * (A.m - 1))
    {
        const int i = 1 + node_of(t, A.n);
        const Pix<T> p(A, t - (long long)(i - 1) * A.n);
        const T *g = A.g + (long long)i * A.n;
        const T gc = g[p.c];
        const bool ex = A.nodes[i].l[0] != nullptr;
        // p = 0.5 p (g(k+1) + g(k)), or e + that with direction fields
        auto scale = [&](T *f, const T *e, T gn) {
            const T r = mul(mul((T)0.5, *f), add(gn, gc));
            *f = ex ? add(*e, r) : r;
        };
        long long o = (long long)i * A.f1 + i1(A, p.y, p.x, p.z);
        if (p.y + 1 < A.d1)
            scale(A.p1 + o, A.e1 + o, g[p.c + 1]);
        o = (long long)i * A.f2 + i2(A, p.y, p.x, p.z);
        if (p.x + 1 < A.d2)
            scale(A.p2 + o, A.e2 + o, g[p.c + A.d1]);
        o = (long long)i * A.f3 + i3(A, p.y, p.x, p.z);
        if (A.dim == 3 && p.z + 1 < A.d3)
            scale(A.p3 + o, A.e3 + o, g[p.c + (long long)A.d1 * A.d2]);
    }
}

template <class T>
__global__ void k5_divergence(const HArgs<T> A)
{
    H_LOOP(A.n * (A.m - 1))
    {
        const int i = 1 + node_of(t, A.n);
        const Pix<T> p(A, t - (long long)(i - 1) * A.n);
        const T *f1 = A.p1 + (long long)i * A.f1;
        const T *f2 = A.p2 + (long long)i * A.f2;
        const T *f3 = A.p3 + (long long)i * A.f3;
        T d = (p.y + 1 < A.d1) ? f1[i1(A, p.y, p.x, p.z)] : (T)0;
        if (p.y >= 1)
            d = sub(d, f1[i1(A, p.y - 1, p.x, p.z)]);
        if (p.x + 1 < A.d2)
            d = add(d, f2[i2(A, p.y, p.x, p.z)]);
        if (p.x >= 1)
            d = sub(d, f2[i2(A, p.y, p.x - 1, p.z)]);
        if (A.dim == 3) {
            if (p.z + 1 < A.d3)
                d = add(d, f3[i3(A, p.y, p.x, p.z)]);
            if (p.z >= 1)
                d = sub(d, f3[i3(A, p.y, p.x, p.z - 1)]);
        }
        A.div[(long long)i * A.n + p.c] = d;
    }
}

// InitializeFullFlow / InitializePseudoFlow: unit direction vectors, 0 where
// sqrt(lx^2 + ly^2 (+ lz^2)) is at most 0.001 (compared in T).  The DAG
// classes initialise a node once per path from the root (each parent
// recurses into it), and the normalisation is repeated as often.
template <class T>
__global__ void k_norm_dirs(const HArgs<T> A)
{
    H_LOOP(A.n * A.m)
    {
        const int i = node_of(t, A.n);
        const long long c = t - (long long)i * A.n;
        const NodeDev<T> &nd = A.nodes[i];
        T *const *l = nd.l;
        if (!l[0])
            continue;
        T v[3] = {l[0][c], l[1][c], A.dim == 3 ? l[2][c] : (T)0};
        for (int r = 0; r < nd.nnorm; ++r) {
            T s = mul(v[0], v[0]);
            for (int k = 1; k < A.dim; ++k)
                s = add(s, mul(v[k], v[k]));
            const T den = sqr(s);
            const bool keep = den > (T)0.001;
            for (int k = 0; k < A.dim; ++k)
                v[k] = keep ? dvd(v[k], den) : (T)0;
        }
        for (int k = 0; k < A.dim; ++k)
            l[k][c] = v[k];
    }
}

// max((m).*v.*l, 0): x for x > 0, else +0 (NaN gives 0)
template <class T>
__device__ __forceinline__ T pos_part(bool m, T v, T l)
{
    const T x = mul(mul(m ? (T)1 : (T)0, v), l);
    return x > (T)0 ? x : (T)0;
}

// exemption amount a per cell (into g): first axis backward then forward
// (one addition, either order), then each further axis forward, backward
template <class T>
__global__ void k_exempt_a(const HArgs<T> A)
{
    H_LOOP(A.n * (A.m - 1))
    {
        const int i = 1 + node_of(t, A.n);
        T *const *l = A.nodes[i].l;
        if (!l[0])
            continue;
        const Pix<T> p(A, t - (long long)(i - 1) * A.n);
        const T *f1 = A.p1 + (long long)i * A.f1;
        const T *f2 = A.p2 + (long long)i * A.f2;
        const T *f3 = A.p3 + (long long)i * A.f3;
        T a = (T)0;
        if (p.y >= 1) {
            const T v = f1[i1(A, p.y - 1, p.x, p.z)];
            a = add(a, pos_part(v < (T)0, v, l[0][p.c]));
        }
        if (p.y + 1 < A.d1) {
            const T v = f1[i1(A, p.y, p.x, p.z)];
            a = add(a, pos_part(v > (T)0, v, l[0][p.c]));
        }
        if (p.x + 1 < A.d2) {
            const T v = f2[i2(A, p.y, p.x, p.z)];
            a = add(a, pos_part(v > (T)0, v, l[1][p.c]));
        }
        if (p.x >= 1) {
            const T v = f2[i2(A, p.y, p.x - 1, p.z)];
            a = add(a, pos_part(v < (T)0, v, l[1][p.c]));
        }
        if (A.dim == 3) {
            if (p.z + 1 < A.d3) {
                const T v = f3[i3(A, p.y, p.x, p.z)];
                a = add(a, pos_part(v > (T)0, v, l[2][p.c]));
            }
            if (p.z >= 1) {
                const T v = f3[i3(A, p.y, p.x, p.z - 1)];
                a = add(a, pos_part(v < (T)0, v, l[2][p.c]));
            }
        }
        A.g[(long long)i * A.n + p.c] = a;
    }
}

// exempt flow of each forward face: the part along the direction of the cell
// it leaves, e = (p>0 & l(k)>0) l(k) a(k) + (p<0 & l(k+1)<0) l(k+1) a(k+1);
// the flow keeps p - e until the rescale adds e back
template <class T>
__global__ void k_exempt_e(const HArgs<T> A)
{
    H_LOOP(A.n * (A.m - 1))
    {
        const int i = 1 + node_of(t, A.n);
        T *const *l = A.nodes[i].l;
        if (!l[0])
            continue;
        const Pix<T> p(A, t - (long long)(i - 1) * A.n);
        const T *a = A.g + (long long)i * A.n;
        auto face = [&](T *f, T *e, const T *lk, long long step) {
            const T v = *f;
            const T llo = lk[p.c], lhi = lk[p.c + step];
            T x = mul(mul((v > (T)0 && llo > (T)0) ? (T)1 : (T)0, llo), a[p.c]);
            x = add(x, mul(mul((v < (T)0 && lhi < (T)0) ? (T)1 : (T)0, lhi), a[p.c + step]));
            *e = x;
            *f = sub(v, x);
        };
        long long o = (long long)i * A.f1 + i1(A, p.y, p.x, p.z);
        if (p.y + 1 < A.d1)
            face(A.p1 + o, A.e1 + o, l[0], 1);
        o = (long long)i * A.f2 + i2(A, p.y, p.x, p.z);
        if (p.x + 1 < A.d2)
            face(A.p2 + o, A.e2 + o, l[1], A.d1);
        o = (long long)i * A.f3 + i3(A, p.y, p.x, p.z);
        if (A.dim == 3 && p.z + 1 < A.d3)
            face(A.p3 + o, A.e3 + o, l[2], (long long)A.d1 * A.d2);
    }
}

// MaxPseudoFlow, per pixel: ResetPseudoFlowCapacity, PushDownPseudoFlows,
// UpdatePseudoFlowLabels (the root's g sums the leaves' labels),
// NormalizePseudoFlowLabels, PushUpCapacityReqs, and steps*g of every
// non-root node (UpdateSpatialPseudoFlows' first line).
template <class T>
__global__ void k_pseudo_point(const HArgs<T> A)
{
    H_LOOP(A.n)
    {
        const long long c = t;
        T *g = A.g + c;
        T *u = A.u + c;
        const long long n = A.n;
        for (int i = 0; i < A.m; ++i) {
            const NodeDev<T> &nd = A.nodes[i];
            g[i * n] = nd.nchild == 0 ? add(A.div[i * n + c], nd.ct[c]) : (T)0;
        }
        for (int i = 0; i < A.m; ++i) {
            const NodeDev<T> &nd = A.nodes[i];
            for (int j = 0; j < nd.nchild; ++j) {
                const long long oc = (long long)A.children[nd.child_begin + j] * n;
                g[oc] = add(g[oc], g[i * n]);
            }
        }
        T acc = (T)0;
        for (int i = 0; i < A.m; ++i) {
            if (A.nodes[i].nchild != 0)
                continue;
            const T v = mul(u[i * n], expo(dvd(-g[i * n], A.cc)));
            u[i * n] = v;
            g[i * n] = v;
            acc = add(acc, v);
        }
        for (int i = 0; i < A.m; ++i) {
            if (A.nodes[i].nchild != 0)
                continue;
            T v = dvd(u[i * n], acc);
            if (v > (T)1)
                v = (T)1;
            if (v < (T)0)
                v = (T)0;
            u[i * n] = v;
        }
        for (int i = A.m - 1; i >= 1; --i) {
            const NodeDev<T> &nd = A.nodes[i];
            if (nd.nchild == 0)
                continue;
            T s = (T)0;
            for (int j = 0; j < nd.nchild; ++j)
                s = add(s, g[(long long)A.children[nd.child_begin + j] * n]);
            g[i * n] = s;
        }
        g[0] = (T)0;
        for (int i = 1; i < A.m; ++i)
            g[i * n] = mul(A.steps, g[i * n]);
    }
}

// DeInitializePseudoFlow: an inner node's u is the sum of its children's
template <class T>
__global__ void k_pseudo_final(const HArgs<T> A)
{
    H_LOOP(A.n)
    {
        T *u = A.u + t;
        for (int i = A.m - 1; i >= 0; --i) {
            const NodeDev<T> &nd = A.nodes[i];
            if (nd.nchild == 0)
                continue;
            T s = u[(long long)A.children[nd.child_begin] * A.n];
            for (int j = 1; j < nd.nchild; ++j)
                s = add(s, u[(long long)A.children[nd.child_begin + j] * A.n]);
            u[(long long)i * A.n] = s;
        }
    }
}

// CalculateCostsFullFlow: sum u*Ct (leaves) and sum u*div (below the root)
// per node.  Block (x, i) sums a stripe of node i's pixels, then adds its
// two partial sums (one atomic pair per block).
template <class T>
__global__ void k_costs(const HArgs<T> A)
{
    __shared__ double s_red[2][kThreads / 32];
    const int i = blockIdx.y;
    const bool leaf = A.nodes[i].nchild == 0, below_root = A.nodes[i].parent >= 0;
    const T *ct = A.nodes[i].ct;
    const T *u = A.u + (long long)i * A.n, *dv = A.div + (long long)i * A.n;
    double dc = 0.0, rc = 0.0;
    for (long long c = blockIdx.x * (long long)kThreads + threadIdx.x; c < A.n;
         c += (long long)gridDim.x * kThreads) {
        const double uc = (double)u[c];
        if (leaf)
            dc += uc * (double)ct[c];
        if (below_root)
            rc += uc * (double)dv[c];
    }
    for (int o = 16; o > 0; o >>= 1) {
        dc += __shfl_xor_sync(0xffffffffu, dc, o);
        rc += __shfl_xor_sync(0xffffffffu, rc, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s_red[0][threadIdx.x >> 5] = dc;
        s_red[1][threadIdx.x >> 5] = rc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kThreads / 32; ++w) {
            dc += s_red[0][w];
            rc += s_red[1][w];
        }
        if (leaf)
            atomicAdd(&A.cost[2 * i], dc);
        if (below_root)
            atomicAdd(&A.cost[2 * i + 1], rc);
    }
}

// ---------------------------------------------------------------- DAG
template <class T>
__device__ __forceinline__ T dag_in(const HArgs<T> &A, const NodeDev<T> &nd, int i, long long c)
{
    return nd.nparent > 1 ? A.pn[(long long)i * A.n + c] : A.pt[(long long)nd.parent * A.n + c];
}

// InitializeFullFlow: pt = Ct (leaves) or max(0, pt of the first child);
// pn = pt (2D) or 0 (3D) for nodes with several parents.
template <class T>
__global__ void k_dag_init(const HArgs<T> A)
{
    H_LOOP(A.n)
    {
        for (int j = A.m - 1; j >= 0; --j) {
            const int i = A.order[j];
            const NodeDev<T> nd = A.nodes[i];
            const long long o = (long long)i * A.n + t;
            T pt;
            if (nd.nchild == 0) {
                pt = nd.ct[t];
            } else {
                const T x = A.pt[(long long)A.children[nd.child_begin] * A.n + t];
                const T z = (T)0;
                pt = (z >= x) ? z : x;
            }
            A.pt[o] = pt;
            if (nd.nparent > 1)
                A.pn[o] = A.dim == 2 ? pt : (T)0;
        }
    }
}

// UpdateSpatialFlows' first line: g = steps*(div + pt - in - u/cc)
template <class T>
__global__ void k_dag_g(const HArgs<T> A)
{
    H_LOOP(A.n * (A.m - 1))
    {
        const int i = 1 + node_of(t, A.n);
        const long long c = t - (long long)(i - 1) * A.n;
        const long long o = (long long)i * A.n + c;
        const T in = dag_in(A, A.nodes[i], i, c);
        A.g[o] = mul(A.steps, sub(sub(add(A.div[o], A.pt[o]), in), dvd(A.u[o], A.cc)));
    }
}

// pn reset, PushDownFlows (top-down), PushCapacityUp (bottom-up), labels.
template <class T>
__global__ void k_dag_point(const HArgs<T> A)
{
    H_LOOP(A.n)
    {
        const long long c = t;
        for (int i = 0; i < A.m; ++i)
            if (A.nodes[i].nparent > 1)
                A.pn[(long long)i * A.n + c] = (T)0;
        for (int j = 0; j < A.m; ++j) {
            const int i = A.order[j];
            const NodeDev<T> nd = A.nodes[i];
            const long long o = (long long)i * A.n + c;
            const T pt = A.pt[o];
            for (int k = 0; k < nd.nchild; ++k) {
                const int ch = A.children[nd.child_begin + k];
                if (A.nodes[ch].nparent > 1) {
                    T *pn = A.pn + (long long)ch * A.n + c;
                    *pn = add(*pn, mul(A.wchild[nd.child_begin + k], pt));
                }
            }
            if (nd.nparent > 0 && nd.nchild > 0)
                A.g[o] = add(sub(dag_in(A, nd, i, c), A.div[o]), dvd(A.u[o], A.cc));
            else if (nd.nparent == 0)
                A.g[o] = A.inv_cc;
        }
        for (int j = A.m - 1; j >= 0; --j) {
            const int i = A.order[j];
            const NodeDev<T> nd = A.nodes[i];
            const long long o = (long long)i * A.n + c;
            if (nd.nchild == 0) {
                const T x = add(sub(dag_in(A, nd, i, c), A.div[o]), dvd(A.u[o], A.cc));
                const T ct = nd.ct[c];
                A.pt[o] = (ct <= x || ct != ct) ? ct : x;
                continue;
            }
            const T pto = A.pt[o];
            T g = A.g[o];
            for (int k = 0; k < nd.nchild; ++k) {
                const int ch = A.children[nd.child_begin + k];
                const long long oc = (long long)ch * A.n + c;
                const T uc = dvd(A.u[oc], A.cc);
                if (A.nodes[ch].nparent > 1) {
                    const T w = A.wchild[nd.child_begin + k];
                    const T e = sub(sub(add(add(A.div[oc], A.pt[oc]), mul(w, pto)), A.pn[oc]), uc);
                    g = add(g, mul(w, e));
                } else {
                    g = sub(add(add(g, A.div[oc]), A.pt[oc]), uc);
                }
            }
            A.g[o] = g;
            A.pt[o] = dvd(g, nd.wdiv);
        }
        for (int j = 0; j < A.m; ++j) {
            const int i = A.order[j];
            const NodeDev<T> nd = A.nodes[i];
            if (nd.nparent == 0)
                continue;
            const long long o = (long long)i * A.n + c;
            A.u[o] = add(A.u[o], mul(A.cc, sub(sub(dag_in(A, nd, i, c), A.div[o]), A.pt[o])));
        }
    }
}

// k_dag_point with the pixel's values of every node staged in shared memory
// (one column per thread; as k1_staged): sink flow (a leaf's slot holds Ct
// until its update, its old sink flow is never read), divergence, label,
// pushed-down flow and the gradient input, with the graph's tables staged
// once per block.  Same operations in the same order as k_dag_point; pn, g
// and u are stored for the nodes k_dag_point stores them for.
struct DagStage {
    // ints: parent count, first parent, first child, child count, the
    // top-down order (5m) and the children list (E); then the weights: wdiv
    // (m) and the child edges' (E); then the nodes' Ct pointers; then the
    // five per-thread columns of every node
    __host__ __device__ static constexpr int int_bytes(int m, int e) { return (4 * (5 * m + e) + 15) / 16 * 16; }
    __host__ __device__ static constexpr int w_bytes(int m, int e, int elem) { return (elem * (m + e) + 15) / 16 * 16; }
    __host__ __device__ static constexpr int table_bytes(int m, int e, int elem)
    {
        return int_bytes(m, e) + w_bytes(m, e, elem) + (8 * m + 15) / 16 * 16;
    }
    __host__ __device__ static constexpr int bytes(int m, int e, int elem)
    {
        return table_bytes(m, e, elem) + 5 * m * kThreads * elem;
    }
};

template <class T>
__global__ void __launch_bounds__(kThreads) k_dag_point_staged(const HArgs<T> A)
{
    extern __shared__ __align__(16) unsigned char dsm[];
    const int m = A.m, ne = A.nedges, tid = threadIdx.x;
    int *npar = reinterpret_cast<int *>(dsm);
    int *par = npar + m, *first = par + m, *cnt = first + m, *order = cnt + m, *kids = order + m;
    T *wdiv = reinterpret_cast<T *>(dsm + DagStage::int_bytes(m, ne));
    T *wch = wdiv + m;
    const T **cts = reinterpret_cast<const T **>(dsm + DagStage::int_bytes(m, ne) +
                                                 DagStage::w_bytes(m, ne, (int)sizeof(T)));
    T *PT = reinterpret_cast<T *>(dsm + DagStage::table_bytes(m, ne, (int)sizeof(T)));
    T *DV = PT + m * kThreads, *U = DV + m * kThreads, *PN = U + m * kThreads, *G = PN + m * kThreads;
    for (int i = tid; i < m; i += kThreads) {
        const NodeDev<T> &nd = A.nodes[i];
        npar[i] = nd.nparent;
        par[i] = nd.parent;
        first[i] = nd.child_begin;
        cnt[i] = nd.nchild;
        order[i] = A.order[i];
        wdiv[i] = nd.wdiv;
        cts[i] = nd.ct;
    }
    for (int j = tid; j < ne; j += kThreads) {
        kids[j] = A.children[j];
        wch[j] = A.wchild[j];
    }
    __syncthreads();
    auto col = [&](T *X, int i) -> T & { return X[i * kThreads + tid]; };
    // flow into node i: its pushed-down flow, or its one parent's sink flow
    auto in_of = [&](int i) -> T { return npar[i] > 1 ? col(PN, i) : col(PT, par[i]); };
    H_LOOP(A.n)
    {
        const long long c = t;
        for (int i = 0; i < m; ++i) {
            const long long o = (long long)i * A.n + c;
            col(PT, i) = cnt[i] == 0 ? cts[i][c] : A.pt[o];
            col(DV, i) = A.div[o];
            col(U, i) = A.u[o];
            col(PN, i) = (T)0;
        }
        // PushDownFlows, top-down
        for (int j = 0; j < m; ++j) {
            const int i = order[j];
            const T pt = col(PT, i);
            for (int k = 0; k < cnt[i]; ++k) {
                const int ch = kids[first[i] + k];
                if (npar[ch] > 1)
                    col(PN, ch) = add(col(PN, ch), mul(wch[first[i] + k], pt));
            }
            if (npar[i] > 0 && cnt[i] > 0)
                col(G, i) = add(sub(in_of(i), col(DV, i)), dvd(col(U, i), A.cc));
            else if (npar[i] == 0)
                col(G, i) = A.inv_cc;
        }
        // PushCapacityUp, bottom-up
        for (int j = m - 1; j >= 0; --j) {
            const int i = order[j];
            if (cnt[i] == 0) {
                const T x = add(sub(in_of(i), col(DV, i)), dvd(col(U, i), A.cc));
                const T ct = col(PT, i);
                col(PT, i) = (ct <= x || ct != ct) ? ct : x;
                continue;
            }
            const T pto = col(PT, i);
            T g = col(G, i);
            for (int k = 0; k < cnt[i]; ++k) {
                const int ch = kids[first[i] + k];
                const T uc = dvd(col(U, ch), A.cc);
                if (npar[ch] > 1) {
                    const T w = wch[first[i] + k];
                    const T e = sub(sub(add(add(col(DV, ch), col(PT, ch)), mul(w, pto)), col(PN, ch)), uc);
                    g = add(g, mul(w, e));
                } else {
                    g = sub(add(add(g, col(DV, ch)), col(PT, ch)), uc);
                }
            }
            col(G, i) = g;
            col(PT, i) = dvd(g, wdiv[i]);
        }
        // labels, top-down
        for (int j = 0; j < m; ++j) {
            const int i = order[j];
            if (npar[i] == 0)
                continue;
            col(U, i) = add(col(U, i), mul(A.cc, sub(sub(in_of(i), col(DV, i)), col(PT, i))));
        }
        for (int i = 0; i < m; ++i) {
            const long long o = (long long)i * A.n + c;
            A.pt[o] = col(PT, i);
            if (npar[i] > 0)
                A.u[o] = col(U, i);
            if (npar[i] > 1)
                A.pn[o] = col(PN, i);
            if (cnt[i] > 0)
                A.g[o] = col(G, i);
        }
    }
}

// The four spatial passes (k2 .. k5) fused for 2D solves without direction
// fields: one block per (node, R x S tile of cells) computes, in shared
// memory over the tile and a two-cell halo, the gradient step of the faces
// (k2), the projection factor (k3), the rescale (k4) and the divergence
// (k5), with each pass's expression and validity tests, and stores the
// tile's faces, divergence and factor (g) as the passes leave them.  The
// halo's faces are recomputed by the neighbouring tiles' blocks; one read
// and one write of each array instead of four passes over them.  The frame
// is R + 4 = 32 rows high: lane q of every warp owns frame row q (y0 - 2 +
// q) in every phase, and warp w the frame columns w, w + 8, ..., so a
// thread's row tests are made once and a warp's loads and stores are one
// 128-byte run of a column.
template <class T, int R, int S>
struct SpatialTile {
    static constexpr int FR = R + 4;   // frame cells y0-2 .. y0+R+1
    static constexpr int FC = S + 4;   // frame cells x0-2 .. x0+S+1
    static constexpr int F = FR * FC;
    static_assert(FR == 32, "one frame row per lane");
    static constexpr int smem_bytes() { return 5 * F * (int)sizeof(T); }
};

template <class T, int R, int S>
__global__ void __launch_bounds__(kThreads) k_spatial_tile2d(const HArgs<T> A, int tiles_y)
{
    using Q = SpatialTile<T, R, S>;
    constexpr int FR = Q::FR, FC = Q::FC, F = Q::F, NW = kThreads / 32;
    extern __shared__ __align__(16) unsigned char hsm[];
    T *G = reinterpret_cast<T *>(hsm);   // g, at cells
    T *P1 = G + F;                        // face (y, y+1) at cell y
    T *P2 = P1 + F;                       // face (x, x+1) at cell x
    T *FS = P2 + F;                       // projection factor
    T *AL = FS + F;
    const int i = 1 + (int)blockIdx.y;    // non-root node
    const int y0 = ((int)blockIdx.x % tiles_y) * R, x0 = ((int)blockIdx.x / tiles_y) * S;
    const int d1 = A.d1, d2 = A.d2;
    const NodeDev<T> nd = A.nodes[i];
    const T *g = A.g + (long long)i * A.n;
    T *p1 = A.p1 + (long long)i * A.f1;
    T *p2 = A.p2 + (long long)i * A.f2;
    const int q = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int y = y0 - 2 + q;
    const bool y_in = (y >= 0 && y < d1), y_up = (y + 1 < d1), y_dn = (y >= 1);
    for (int c = w; c < FC; c += NW) {
        const int x = x0 - 2 + c, f = c * FR + q;
        const bool in = y_in && x >= 0 && x < d2;
        const unsigned int cell = (unsigned int)x * (unsigned int)d1 + (unsigned int)y;
        G[f] = in ? g[cell] : (T)0;
        P1[f] = (in && y_up) ? p1[(unsigned int)x * (unsigned int)(d1 - 1) + (unsigned int)y] : (T)0;
        P2[f] = (in && x + 1 < d2) ? p2[cell] : (T)0;
        AL[f] = in ? (nd.alpha ? nd.alpha[cell] : nd.alpha_s) : (T)0;
    }
    __syncthreads();
    // k2: 2D p + (g(k+1) - g(k)) (asetsHMF2D.m), else (p + g(k+1)) - g(k)
    auto step = [&](T pv, T gn, T gc) { return A.paren ? add(pv, sub(gn, gc)) : sub(add(pv, gn), gc); };
    if (q <= R + 2 && y_in && y_up) {                            // p1: y0-2 .. y0+R, x0-1 .. x0+S
        for (int c = 1 + w; c <= S + 2; c += NW) {
            const int x = x0 - 2 + c, f = c * FR + q;
            if (x >= 0 && x < d2)
                P1[f] = step(P1[f], G[f + 1], G[f]);
        }
    }
    if (q >= 1 && q <= R + 2 && y_in) {                          // p2: y0-1 .. y0+R, x0-2 .. x0+S
        for (int c = w; c <= S + 2; c += NW) {
            const int x = x0 - 2 + c, f = c * FR + q;
            if (x >= 0 && x + 1 < d2)
                P2[f] = step(P2[f], G[f + FR], G[f]);
        }
    }
    __syncthreads();
    // k3: the cell's faces' squares in the .m files' order, the factor
    if (q >= 1 && q <= R + 2 && y_in) {                          // y0-1 .. y0+R, x0-1 .. x0+S
        for (int c = 1 + w; c <= S + 2; c += NW) {
            const int x = x0 - 2 + c, f = c * FR + q;
            if (x < 0 || x >= d2)
                continue;
            T sq = (T)0;
            if (y_up)
                sq = add(sq, mul(P1[f], P1[f]));
            if (y_dn)
                sq = add(sq, mul(P1[f - 1], P1[f - 1]));
            if (x + 1 < d2)
                sq = add(sq, mul(P2[f], P2[f]));
            if (x >= 1)
                sq = add(sq, mul(P2[f - FR], P2[f - FR]));
            const T mag = sqr(sq);
            const T al = AL[f];
            FS[f] = (mag <= al) ? (T)1 : dvd(al, mag);
        }
    }
    __syncthreads();
    // k4: p = 0.5 p (f(k+1) + f(k)); the tile's own faces are stored
    if (q >= 1 && q <= R + 1 && y >= 0 && y_up) {                // p1: y0-1 .. y0+R-1, tile columns
        for (int c = 2 + w; c <= S + 1; c += NW) {
            const int x = x0 - 2 + c, f = c * FR + q;
            if (x >= d2)
                break;
            const T r = mul(mul((T)0.5, P1[f]), add(FS[f + 1], FS[f]));
            P1[f] = r;
            if (q >= 2)
                p1[(unsigned int)x * (unsigned int)(d1 - 1) + (unsigned int)y] = r;
        }
    }
    if (q >= 2 && q <= R + 1 && y < d1) {                        // p2: tile rows, x0-1 .. x0+S-1
        for (int c = 1 + w; c <= S + 1; c += NW) {
            const int x = x0 - 2 + c, f = c * FR + q;
            if (x + 1 >= d2)
                break;
            if (x < 0)
                continue;
            const T r = mul(mul((T)0.5, P2[f]), add(FS[f + FR], FS[f]));
            P2[f] = r;
            if (c >= 2)
                p2[(unsigned int)x * (unsigned int)d1 + (unsigned int)y] = r;
        }
    }
    __syncthreads();
    // k5: the tile's divergence; g keeps the factor, as k3 leaves it
    T *divp = A.div + (long long)i * A.n;
    T *gw = A.g + (long long)i * A.n;
    if (q >= 2 && q <= R + 1 && y < d1) {
        for (int c = 2 + w; c <= S + 1; c += NW) {
            const int x = x0 - 2 + c, f = c * FR + q;
            if (x >= d2)
                break;
            T d = y_up ? P1[f] : (T)0;
            if (y_dn)
                d = sub(d, P1[f - 1]);
            if (x + 1 < d2)
                d = add(d, P2[f]);
            if (x >= 1)
                d = sub(d, P2[f - FR]);
            const unsigned int cell = (unsigned int)x * (unsigned int)d1 + (unsigned int)y;
            divp[cell] = d;
            gw[cell] = FS[f];
        }
    }
}

int h_grid(long long n, int sms)
{
    long long b = (n + kThreads - 1) / kThreads;
    const long long cap = (long long)sms * 8;
    return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

// gradient step on g, the geodesic exemption (nodes with direction fields),
// flow magnitude and projection factor, rescale, divergence
template <class T>
void spatial_passes(const HArgs<T> &A, int gn, cudaStream_t st, bool dirs)
{
    if (A.dim == 2 && !dirs && A.m > 1) {
        // 28 x 32 tiles: a 32-row frame (one row per lane), within the
        // default 48 KB of dynamic shared memory in double as well
        constexpr int R = 28, S = 32;
        using Q = SpatialTile<T, R, S>;
        static_assert(Q::smem_bytes() <= 48 * 1024, "frame above the default shared memory");
        const int ty = (A.d1 + R - 1) / R, tx = (A.d2 + S - 1) / S;
        k_spatial_tile2d<T, R, S><<<dim3(ty * tx, A.m - 1), kThreads, Q::smem_bytes(), st>>>(A, ty);
        return;
    }
    k2_gradient<T><<<gn, kThreads, 0, st>>>(A);
    if (dirs) {
        k_exempt_a<T><<<gn, kThreads, 0, st>>>(A);
        k_exempt_e<T><<<gn, kThreads, 0, st>>>(A);
    }
    k3_projection<T><<<gn, kThreads, 0, st>>>(A);
    k4_rescale<T><<<gn, kThreads, 0, st>>>(A);
    k5_divergence<T><<<gn, kThreads, 0, st>>>(A);
}

// Device copies of the nodes' direction fields (ld[k][i], host, null for a
// node without) and the exempt-flow buffers; false when out of memory.
template <class T, class Get>
bool setup_dirs(Get &get, cudaStream_t st, int dim, int m, void *const *const ld[3],
                std::vector<NodeDev<T>> &nodes, HArgs<T> &A, cudaError_t &e, bool &any)
{
    any = false;
    for (int i = 0; i < m; ++i) {
        if (!ld[0] || !ld[0][i])
            continue;
        any = true;
        void *vp = nullptr;
        if (!get(&vp, sizeof(T) * A.n * dim))
            return false;
        for (int k = 0; k < dim; ++k) {
            nodes[i].l[k] = static_cast<T *>(vp) + A.n * k;
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(nodes[i].l[k], ld[k][i], sizeof(T) * A.n, cudaMemcpyHostToDevice, st);
        }
    }
    if (any) {
        void *vp = nullptr;
        if (!get(&vp, sizeof(T) * (A.f1 + A.f2 + A.f3) * m))
            return false;
        A.e1 = static_cast<T *>(vp);
        A.e2 = A.e1 + A.f1 * m;
        A.e3 = A.e2 + A.f2 * m;
    }
    return true;
}

// the normalised direction fields back into the caller's arrays
template <class T>
cudaError_t download_dirs(cudaStream_t st, int dim, int m, long long n, void *const *const ld[3],
                          const std::vector<NodeDev<T>> &nodes)
{
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < m && e == cudaSuccess; ++i)
        for (int k = 0; k < dim && e == cudaSuccess && nodes[i].l[0]; ++k)
            e = cudaMemcpyAsync(ld[k][i], nodes[i].l[k], sizeof(T) * n, cudaMemcpyDeviceToHost, st);
    return e;
}

template <class T>
asets_status run_hmf(asets_context *ctx, int algo, int dim, int d1, int d2, int d3, int m,
                     const int *parent, const void *const *Ct, const void *const *alpha_arr,
                     const double *alpha_s, void *const *const ld[3], int its, double steps,
                     double cc, void *const *u_out, void *const *pt_out, void *const *div_out,
                     void *const *g_out, void *const *p_out[3], double *data_cost,
                     double *regu_cost)
{
    const bool pseudo = (algo == ASETS_HMF_PSEUDO_FLOW);
    cudaStream_t st = context_stream(ctx);
    const int sms = context_num_sms(ctx);
    const long long n = (long long)d1 * d2 * d3;
    const long long f1 = (long long)(d1 - 1) * d2 * d3, f2 = (long long)d1 * (d2 - 1) * d3,
                    f3 = dim == 3 ? (long long)d1 * d2 * (d3 - 1) : 0;
    // tree tables (children of each node in index order)
    std::vector<int> nchild(m, 0), begin(m, 0), kids;
    for (int i = 1; i < m; ++i)
        ++nchild[parent[i]];
    for (int i = 0, acc = 0; i < m; ++i) {
        begin[i] = acc;
        acc += nchild[i];
    }
    kids.assign(m > 1 ? m - 1 : 1, 0);
    {
        std::vector<int> fill(begin);
        for (int i = 1; i < m; ++i)
            kids[fill[parent[i]]++] = i;
    }
    std::vector<void *> bufs;
    asets_status status = ASETS_OK;
    auto get = [&](void **p, size_t bytes) {
        if (cudaMallocAsync(p, bytes ? bytes : 8, st) != cudaSuccess)
            return false;
        bufs.push_back(*p);
        return true;
    };
    HArgs<T> A;
    memset(&A, 0, sizeof A);
    A.dim = dim;
    A.d1 = d1;
    A.d2 = d2;
    A.d3 = d3;
    A.m = m;
    A.n = n;
    A.f1 = f1;
    A.f2 = f2;
    A.f3 = f3;
    A.cc = (T)cc;
    A.steps = (T)steps;
    A.inv_cc = (T)(1.0 / cc);
    // asetsHMF2D.m parenthesises the full-flow gradient step, not the pseudo-flow one
    A.paren = (dim == 2 && !pseudo) ? 1 : 0;
    std::vector<NodeDev<T>> nodes(m);
    void *vp = nullptr;
    cudaError_t e = cudaSuccess;
    bool ok = get(&vp, sizeof(T) * n * m * 4);
    if (ok) {
        T *base = static_cast<T *>(vp);
        A.pt = base;
        A.u = base + n * m;
        A.div = base + 2 * n * m;
        A.g = base + 3 * n * m;
        e = cudaMemsetAsync(vp, 0, sizeof(T) * n * m * 4, st);
    }
    const long long fsum = (f1 + f2 + f3) * m;
    ok = ok && get(&vp, sizeof(T) * fsum);
    if (ok) {
        A.p1 = static_cast<T *>(vp);
        A.p2 = A.p1 + f1 * m;
        A.p3 = A.p2 + f2 * m;
        if (e == cudaSuccess)
            e = cudaMemsetAsync(vp, 0, sizeof(T) * fsum, st);
    }
    ok = ok && get(&vp, sizeof(double) * 2 * m);
    if (ok) {
        A.cost = static_cast<double *>(vp);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(vp, 0, sizeof(double) * 2 * m, st);
    }
    for (int i = 0; ok && i < m; ++i) {
        NodeDev<T> &nd = nodes[i];
        nd.parent = parent[i];
        nd.child_begin = begin[i];
        nd.nchild = nchild[i];
        nd.alpha_s = (T)(alpha_s ? alpha_s[i] : 0.0);
        nd.ct = nullptr;
        nd.alpha = nullptr;
        nd.nnorm = 1;
        if (nchild[i] == 0 && e == cudaSuccess) {
            ok = get(&vp, sizeof(T) * n);
            if (ok) {
                e = cudaMemcpyAsync(vp, Ct[i], sizeof(T) * n, cudaMemcpyHostToDevice, st);
                nd.ct = static_cast<const T *>(vp);
            }
        }
        if (ok && alpha_arr && alpha_arr[i] && e == cudaSuccess) {
            ok = get(&vp, sizeof(T) * n);
            if (ok) {
                e = cudaMemcpyAsync(vp, alpha_arr[i], sizeof(T) * n, cudaMemcpyHostToDevice, st);
                nd.alpha = static_cast<const T *>(vp);
            }
        }
        // pseudo-flow starts from the leaves' labels
        if (ok && pseudo && nchild[i] == 0 && e == cudaSuccess)
            e = cudaMemcpyAsync(A.u + (long long)i * n, u_out[i], sizeof(T) * n, cudaMemcpyHostToDevice, st);
    }
    bool dirs = false;
    ok = ok && setup_dirs<T>(get, st, dim, m, ld, nodes, A, e, dirs);
    ok = ok && get(&vp, sizeof(NodeDev<T>) * m);
    if (ok && e == cudaSuccess) {
        e = cudaMemcpyAsync(vp, nodes.data(), sizeof(NodeDev<T>) * m, cudaMemcpyHostToDevice, st);
        A.nodes = static_cast<const NodeDev<T> *>(vp);
    }
    ok = ok && get(&vp, sizeof(int) * kids.size());
    if (ok && e == cudaSuccess) {
        e = cudaMemcpyAsync(vp, kids.data(), sizeof(int) * kids.size(), cudaMemcpyHostToDevice, st);
        A.children = static_cast<const int *>(vp);
    }
    if (!ok) {
        status = ASETS_ERR_OUT_OF_MEMORY;
        set_last_error("asets_hmf_full_flow: out of device memory");
    } else if (e == cudaSuccess) {
        const int gp = h_grid(n, sms), gn = h_grid(n * (m - 1), sms);
        // the staged per-pixel pass for trees whose columns fit the default
        // 48 KB of shared memory (15 nodes in float, 7 in double)
        const int k1_smem = K1Stage::bytes(m, (int)sizeof(T));
        if (dirs)
            k_norm_dirs<T><<<h_grid(n * m, sms), kThreads, 0, st>>>(A);
        for (int it = 0; it < its && e == cudaSuccess; ++it) {
            if (pseudo)
                k_pseudo_point<T><<<gp, kThreads, 0, st>>>(A);
            else if (k1_smem <= 48 * 1024)
                k1_staged<T><<<gp, kThreads, k1_smem, st>>>(A);
            else
                k1_pointwise<T><<<gp, kThreads, 0, st>>>(A);
            spatial_passes(A, gn, st, dirs);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
            if (pseudo)
                k_pseudo_final<T><<<gp, kThreads, 0, st>>>(A);
            else
                k_costs<T><<<dim3(h_grid(n, sms), m), kThreads, 0, st>>>(A);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess && dirs)
            e = download_dirs<T>(st, dim, m, n, ld, nodes);
        std::vector<double> cost(2 * m, 0.0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(cost.data(), A.cost, sizeof(double) * 2 * m, cudaMemcpyDeviceToHost, st);
        for (int i = 0; i < m && e == cudaSuccess; ++i) {
            const size_t nb = sizeof(T) * n;
            if (u_out && u_out[i])
                e = cudaMemcpyAsync(u_out[i], A.u + (long long)i * n, nb, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess && pt_out && pt_out[i] && !pseudo)
                e = cudaMemcpyAsync(pt_out[i], A.pt + (long long)i * n, nb, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess && div_out && div_out[i])
                e = cudaMemcpyAsync(div_out[i], A.div + (long long)i * n, nb, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess && g_out && g_out[i])
                e = cudaMemcpyAsync(g_out[i], A.g + (long long)i * n, nb, cudaMemcpyDeviceToHost, st);
            const T *fp[3] = {A.p1 + f1 * i, A.p2 + f2 * i, A.p3 + f3 * i};
            const long long fn[3] = {f1, f2, f3};
            for (int k = 0; k < dim && e == cudaSuccess; ++k)
                if (p_out[k] && p_out[k][i] && fn[k] > 0)
                    e = cudaMemcpyAsync(p_out[k][i], fp[k], sizeof(T) * fn[k], cudaMemcpyDeviceToHost, st);
        }
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
        if (e == cudaSuccess && !pseudo) {
            // CalculateCostsFullFlow: each node adds its children's costs
            std::vector<double> dc(m), rc(m);
            for (int i = m - 1; i >= 0; --i) {
                dc[i] = cost[2 * i];
                rc[i] = cost[2 * i + 1];
                for (int j = 0; j < nchild[i]; ++j) {
                    dc[i] += dc[kids[begin[i] + j]];
                    rc[i] += rc[kids[begin[i] + j]];
                }
            }
            for (int i = 0; i < m; ++i) {
                if (data_cost)
                    data_cost[i] = dc[i];
                if (regu_cost)
                    regu_cost[i] = rc[i];
            }
        }
    }
    if (status == ASETS_OK && e != cudaSuccess) {
        cudaGetLastError();
        status = ASETS_ERR_CUDA;
        set_last_error((std::string("asets_hmf_full_flow: ") + cudaGetErrorString(e)).c_str());
    }
    for (void *p : bufs)
        cudaFreeAsync(p, st);
    cudaStreamSynchronize(st);
    return status;
}

template <class T>
asets_status run_dag(asets_context *ctx, int dim, int d1, int d2, int d3, int m,
                     const std::vector<int> &nchild, const std::vector<int> &begin,
                     const std::vector<int> &kids, const std::vector<int> &nparent,
                     const std::vector<int> &parent0, const std::vector<int> &order,
                     const void *const *Ct, const void *const *alpha_arr, const double *alpha_s,
                     void *const *const ld[3], int its, double steps, double cc,
                     void *const *outs[5], void *const *p_out[3])
{
    cudaStream_t st = context_stream(ctx);
    const int sms = context_num_sms(ctx);
    const long long n = (long long)d1 * d2 * d3;
    const long long f1 = (long long)(d1 - 1) * d2 * d3, f2 = (long long)d1 * (d2 - 1) * d3,
                    f3 = dim == 3 ? (long long)d1 * d2 * (d3 - 1) : 0;
    std::vector<void *> bufs;
    auto get = [&](void **p, size_t bytes) {
        if (cudaMallocAsync(p, bytes ? bytes : 8, st) != cudaSuccess)
            return false;
        bufs.push_back(*p);
        return true;
    };
    HArgs<T> A;
    memset(&A, 0, sizeof A);
    A.dim = dim;
    A.d1 = d1;
    A.d2 = d2;
    A.d3 = d3;
    A.m = m;
    A.n = n;
    A.f1 = f1;
    A.f2 = f2;
    A.f3 = f3;
    A.cc = (T)cc;
    A.steps = (T)steps;
    A.inv_cc = (T)(1.0 / cc);
    A.paren = 0;  // both DAG files: (p + g(k+1)) - g(k)
    A.nedges = (int)kids.size();
    // child weights 1/(parents of the child); per node the sum of their squares
    std::vector<T> w(kids.size());
    std::vector<NodeDev<T>> nodes(m);
    // paths from the root to each node (the top-down list has parents first),
    // saturating at 2^20
    std::vector<long long> paths(m, 0);
    paths[0] = 1;
    for (int q : order)
        for (int k = 0; k < nchild[q]; ++k) {
            long long &pr = paths[kids[begin[q] + k]];
            pr = std::min(pr + paths[q], 1LL << 20);
        }
    for (int i = 0; i < m; ++i) {
        double s2 = 0.0;
        for (int k = 0; k < nchild[i]; ++k) {
            const double wk = 1.0 / (double)nparent[kids[begin[i] + k]];
            w[begin[i] + k] = (T)wk;
            s2 += wk * wk;
        }
        NodeDev<T> &nd = nodes[i];
        nd.parent = parent0[i];
        nd.nparent = nparent[i];
        nd.child_begin = begin[i];
        nd.nchild = nchild[i];
        nd.wdiv = (T)(nparent[i] == 0 ? s2 : 1.0 + s2);
        nd.nnorm = (int)paths[i];
        nd.alpha_s = (T)(alpha_s ? alpha_s[i] : 0.0);
        nd.ct = nullptr;
        nd.alpha = nullptr;
    }
    cudaError_t e = cudaSuccess;
    void *vp = nullptr;
    bool ok = get(&vp, sizeof(T) * n * m * 5);
    if (ok) {
        T *base = static_cast<T *>(vp);
        A.pt = base;
        A.u = base + n * m;
        A.div = base + 2 * n * m;
        A.g = base + 3 * n * m;
        A.pn = base + 4 * n * m;
        e = cudaMemsetAsync(vp, 0, sizeof(T) * n * m * 5, st);
    }
    const long long fsum = (f1 + f2 + f3) * m;
    ok = ok && get(&vp, sizeof(T) * fsum);
    if (ok) {
        A.p1 = static_cast<T *>(vp);
        A.p2 = A.p1 + f1 * m;
        A.p3 = A.p2 + f2 * m;
        if (e == cudaSuccess)
            e = cudaMemsetAsync(vp, 0, sizeof(T) * fsum, st);
    }
    for (int i = 0; ok && i < m && e == cudaSuccess; ++i) {
        if (nchild[i] == 0) {
            ok = get(&vp, sizeof(T) * n);
            if (ok) {
                e = cudaMemcpyAsync(vp, Ct[i], sizeof(T) * n, cudaMemcpyHostToDevice, st);
                nodes[i].ct = static_cast<const T *>(vp);
            }
        }
        if (ok && e == cudaSuccess && alpha_arr && alpha_arr[i]) {
            ok = get(&vp, sizeof(T) * n);
            if (ok) {
                e = cudaMemcpyAsync(vp, alpha_arr[i], sizeof(T) * n, cudaMemcpyHostToDevice, st);
                nodes[i].alpha = static_cast<const T *>(vp);
            }
        }
    }
    bool dirs = false;
    ok = ok && setup_dirs<T>(get, st, dim, m, ld, nodes, A, e, dirs);
    struct Up {
        const void *src;
        size_t bytes;
        const void **dst;
    } ups[] = {{nodes.data(), sizeof(NodeDev<T>) * m, reinterpret_cast<const void **>(&A.nodes)},
               {kids.data(), sizeof(int) * kids.size(), reinterpret_cast<const void **>(&A.children)},
               {w.data(), sizeof(T) * w.size(), reinterpret_cast<const void **>(&A.wchild)},
               {order.data(), sizeof(int) * order.size(), reinterpret_cast<const void **>(&A.order)}};
    for (auto &u : ups) {
        ok = ok && get(&vp, u.bytes);
        if (ok && e == cudaSuccess) {
            e = cudaMemcpyAsync(vp, u.src, u.bytes, cudaMemcpyHostToDevice, st);
            *u.dst = vp;
        }
    }
    asets_status status = ASETS_OK;
    if (!ok) {
        status = ASETS_ERR_OUT_OF_MEMORY;
        set_last_error("asets_dag_full_flow: out of device memory");
    } else if (e == cudaSuccess) {
        const int gp = h_grid(n, sms), gn = h_grid(n * (m - 1), sms);
        // the staged per-pixel pass for graphs whose columns fit the default
        // 48 KB of shared memory (9 nodes in float, 4 in double)
        const int dag_smem = DagStage::bytes(m, (int)kids.size(), (int)sizeof(T));
        k_dag_init<T><<<gp, kThreads, 0, st>>>(A);
        if (dirs)
            k_norm_dirs<T><<<h_grid(n * m, sms), kThreads, 0, st>>>(A);
        for (int it = 0; it < its && e == cudaSuccess; ++it) {
            k_dag_g<T><<<gn, kThreads, 0, st>>>(A);
            spatial_passes(A, gn, st, dirs);
            if (dag_smem <= 48 * 1024)
                k_dag_point_staged<T><<<gp, kThreads, dag_smem, st>>>(A);
            else
                k_dag_point<T><<<gp, kThreads, 0, st>>>(A);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess && dirs)
            e = download_dirs<T>(st, dim, m, n, ld, nodes);
        T *const srcs[5] = {A.u, A.pt, A.pn, A.div, A.g};
        for (int i = 0; i < m && e == cudaSuccess; ++i) {
            for (int k = 0; k < 5 && e == cudaSuccess; ++k)
                if (outs[k] && outs[k][i])
                    e = cudaMemcpyAsync(outs[k][i], srcs[k] + (long long)i * n, sizeof(T) * n,
                                        cudaMemcpyDeviceToHost, st);
            const T *fp[3] = {A.p1 + f1 * i, A.p2 + f2 * i, A.p3 + f3 * i};
            const long long fn[3] = {f1, f2, f3};
            for (int k = 0; k < dim && e == cudaSuccess; ++k)
                if (p_out[k] && p_out[k][i] && fn[k] > 0)
                    e = cudaMemcpyAsync(p_out[k][i], fp[k], sizeof(T) * fn[k], cudaMemcpyDeviceToHost, st);
        }
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
    }
    if (status == ASETS_OK && e != cudaSuccess) {
        cudaGetLastError();
        status = ASETS_ERR_CUDA;
        set_last_error((std::string("asets_dag_full_flow: ") + cudaGetErrorString(e)).c_str());
    }
    for (void *p : bufs)
        cudaFreeAsync(p, st);
    cudaStreamSynchronize(st);
    return status;
}

// direction fields: a node with lx needs ly (and lz in 3D), as the .m
// files index them unchecked
bool check_dirs(int dim, int m, void *const *const ld[3], const char *fn)
{
    for (int i = 0; ld[0] && i < m; ++i) {
        if (!ld[0][i])
            continue;
        for (int k = 1; k < dim; ++k)
            if (!ld[k] || !ld[k][i]) {
                set_last_error((std::string(fn) + ": a node with lx needs ly (and lz in 3D)").c_str());
                return false;
            }
    }
    return true;
}

}  // namespace

extern "C" ASETS_API asets_status asets_dag_run(
    asets_context *ctx, int precision, int dim, int D1, int D2, int D3, int num_nodes,
    const int *nchild_in, const int *children, const void *const *Ct,
    const void *const *alpha_arrays, const double *alpha_scalars, void *const *lx,
    void *const *ly, void *const *lz, int numIts, double steps, double cc, void *const *u,
    void *const *pt, void *const *pn, void *const *div, void *const *g, void *const *p1,
    void *const *p2, void *const *p3)
{
    void *const *const ld[3] = {lx, ly, lz};
    if (!ctx || !nchild_in || !Ct || (precision != 4 && precision != 8) || (dim != 2 && dim != 3) ||
        D1 < 1 || D2 < 1 || D3 < 1 || (dim == 2 && D3 != 1) || num_nodes < 2 || numIts < 0) {
        set_last_error("asets_dag_full_flow: bad arguments");
        return ASETS_ERR_INVALID_ARG;
    }
    if ((long long)D1 * D2 * D3 * num_nodes >= (1LL << 31)) {
        set_last_error("asets_dag_full_flow: pixels x nodes must stay below 2^31");
        return ASETS_ERR_INVALID_ARG;
    }
    const int m = num_nodes;
    std::vector<int> nchild(nchild_in, nchild_in + m), begin(m, 0), nparent(m, 0), parent0(m, -1);
    int total = 0;
    for (int i = 0; i < m; ++i) {
        if (nchild[i] < 0 || nchild[i] == 1) {
            set_last_error("asets_dag_full_flow: an inner node needs two or more children");
            return ASETS_ERR_INVALID_ARG;
        }
        begin[i] = total;
        total += nchild[i];
    }
    std::vector<int> kids(children ? children : nullptr, children ? children + total : nullptr);
    if ((int)kids.size() != total) {
        set_last_error("asets_dag_full_flow: children missing");
        return ASETS_ERR_INVALID_ARG;
    }
    for (int i = 0; i < m; ++i)
        for (int k = 0; k < nchild[i]; ++k) {
            const int c = kids[begin[i] + k];
            if (c <= 0 || c >= m) {
                set_last_error("asets_dag_full_flow: bad child index (node 0 is the root)");
                return ASETS_ERR_INVALID_ARG;
            }
            if (nparent[c]++ == 0)
                parent0[c] = i;
        }
    if (nparent[0] != 0 || nchild[0] == 0) {
        set_last_error("asets_dag_full_flow: node 0 must be the root, with children");
        return ASETS_ERR_INVALID_ARG;
    }
    for (int i = 0; i < m; ++i)
        if (nchild[i] == 0 && !Ct[i]) {
            set_last_error("asets_dag_full_flow: every leaf needs its Ct");
            return ASETS_ERR_INVALID_ARG;
        }
    if (!check_dirs(dim, m, ld, "asets_dag_full_flow"))
        return ASETS_ERR_INVALID_ARG;
    // the top-down list of MaxFullFlow: depth-first from the root, a node
    // entering the stack once all its parents are listed
    std::vector<int> order, stack{0};
    std::vector<char> listed(m, 0);
    while (!stack.empty()) {
        const int q = stack.back();
        stack.pop_back();
        order.push_back(q);
        listed[q] = 1;
        for (int k = 0; k < nchild[q]; ++k) {
            const int r = kids[begin[q] + k];
            bool all = true;
            for (int i = 0; i < m && all; ++i)
                for (int j = 0; j < nchild[i]; ++j)
                    if (kids[begin[i] + j] == r && !listed[i]) {
                        all = false;
                        break;
                    }
            if (all)
                stack.push_back(r);
        }
    }
    if ((int)order.size() != m) {
        set_last_error("asets_dag_full_flow: the graph has nodes not reachable from the root, or a cycle");
        return ASETS_ERR_INVALID_ARG;
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(context_device(ctx));
    void *const *outs[5] = {u, pt, pn, div, g};
    void *const *p_out[3] = {p1, p2, p3};
    const asets_status s =
        precision == 8
            ? run_dag<double>(ctx, dim, D1, D2, D3, m, nchild, begin, kids, nparent, parent0, order,
                              Ct, alpha_arrays, alpha_scalars, ld, numIts, steps, cc, outs, p_out)
            : run_dag<float>(ctx, dim, D1, D2, D3, m, nchild, begin, kids, nparent, parent0, order,
                             Ct, alpha_arrays, alpha_scalars, ld, numIts, steps, cc, outs, p_out);
    cudaSetDevice(prev);
    return s;
}

extern "C" ASETS_API asets_status asets_dag_full_flow(
    asets_context *ctx, int precision, int dim, int D1, int D2, int D3, int num_nodes,
    const int *nchild, const int *children, const void *const *Ct,
    const void *const *alpha_arrays, const double *alpha_scalars, int numIts, double steps,
    double cc, void *const *u, void *const *pt, void *const *pn, void *const *div,
    void *const *g, void *const *p1, void *const *p2, void *const *p3)
{
    return asets_dag_run(ctx, precision, dim, D1, D2, D3, num_nodes, nchild, children, Ct,
                         alpha_arrays, alpha_scalars, nullptr, nullptr, nullptr, numIts, steps, cc,
                         u, pt, pn, div, g, p1, p2, p3);
}

extern "C" ASETS_API asets_status asets_hmf_run(
    asets_context *ctx, int algorithm, int precision, int dim, int D1, int D2, int D3,
    int num_nodes, const int *parent, const void *const *Ct, const void *const *alpha_arrays,
    const double *alpha_scalars, void *const *lx, void *const *ly, void *const *lz, int numIts,
    double steps, double cc, void *const *u, void *const *pt, void *const *div, void *const *g,
    void *const *p1, void *const *p2, void *const *p3, double *data_cost, double *regu_cost)
{
    void *const *const ld[3] = {lx, ly, lz};
    if (!ctx || !parent || !Ct || (precision != 4 && precision != 8) || (dim != 2 && dim != 3) ||
        D1 < 1 || D2 < 1 || D3 < 1 || (dim == 2 && D3 != 1) || num_nodes < 1 || numIts < 0 ||
        (algorithm != ASETS_HMF_FULL_FLOW && algorithm != ASETS_HMF_PSEUDO_FLOW)) {
        set_last_error("asets_hmf_full_flow: bad arguments");
        return ASETS_ERR_INVALID_ARG;
    }
    if ((long long)D1 * D2 * D3 * num_nodes >= (1LL << 31) || num_nodes > 65535) {
        set_last_error("asets_hmf_full_flow: pixels x nodes must stay below 2^31, nodes below 65536");
        return ASETS_ERR_INVALID_ARG;
    }
    if (parent[0] != -1) {
        set_last_error("asets_hmf_full_flow: node 0 must be the root (parent -1)");
        return ASETS_ERR_INVALID_ARG;
    }
    std::vector<int> nch(num_nodes, 0);
    for (int i = 1; i < num_nodes; ++i) {
        if (parent[i] < 0 || parent[i] >= i) {
            set_last_error("asets_hmf_full_flow: nodes must be in pre-order (parent index < node index)");
            return ASETS_ERR_INVALID_ARG;
        }
        ++nch[parent[i]];
    }
    for (int i = 0; i < num_nodes; ++i)
        if (nch[i] == 0 && !Ct[i]) {
            set_last_error("asets_hmf_full_flow: every leaf needs its Ct");
            return ASETS_ERR_INVALID_ARG;
        }
    if (num_nodes == 1 || nch[0] == 0) {
        set_last_error("asets_hmf_full_flow: the root needs children");
        return ASETS_ERR_INVALID_ARG;
    }
    if (!check_dirs(dim, num_nodes, ld, "asets_hmf_run"))
        return ASETS_ERR_INVALID_ARG;
    if (algorithm == ASETS_HMF_PSEUDO_FLOW)
        for (int i = 0; i < num_nodes; ++i)
            if (nch[i] == 0 && (!u || !u[i])) {
                set_last_error("asets_hmf_run: pseudo-flow reads every leaf's labels from u");
                return ASETS_ERR_INVALID_ARG;
            }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(context_device(ctx));
    void *const *p_out[3] = {p1, p2, p3};
    const asets_status s =
        precision == 8
            ? run_hmf<double>(ctx, algorithm, dim, D1, D2, D3, num_nodes, parent, Ct,
                              alpha_arrays, alpha_scalars, ld, numIts, steps, cc, u, pt, div, g,
                              p_out, data_cost, regu_cost)
            : run_hmf<float>(ctx, algorithm, dim, D1, D2, D3, num_nodes, parent, Ct,
                             alpha_arrays, alpha_scalars, ld, numIts, steps, cc, u, pt, div, g,
                             p_out, data_cost, regu_cost);
    cudaSetDevice(prev);
    return s;
}

extern "C" ASETS_API asets_status asets_hmf_full_flow(
    asets_context *ctx, int precision, int dim, int D1, int D2, int D3, int num_nodes,
    const int *parent, const void *const *Ct, const void *const *alpha_arrays,
    const double *alpha_scalars, int numIts, double steps, double cc, void *const *u,
    void *const *pt, void *const *div, void *const *g, void *const *p1, void *const *p2,
    void *const *p3, double *data_cost, double *regu_cost)
{
    return asets_hmf_run(ctx, ASETS_HMF_FULL_FLOW, precision, dim, D1, D2, D3, num_nodes, parent,
                         Ct, alpha_arrays, alpha_scalars, nullptr, nullptr, nullptr, numIts, steps,
                         cc, u, pt, div, g, p1, p2, p3, data_cost, regu_cost);
}
