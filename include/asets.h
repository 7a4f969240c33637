/*
 * libasetscuda -- GB300 (sm_103a) continuous max-flow solvers.
 *
 * C ABI: plain pointers and sizes, no CUDA or torch types.  Arrays are
 * float32 in Matlab column-major order (index g = z*Nx*Ny + x*Ny + y, the
 * label index slowest), exactly as the reference mex files receive them
 * through mxGetData.
 *
 * Every function returns an asets_status.  On failure nothing is written to
 * the outputs; asets_last_error() gives a message for the calling thread.
 */
#ifndef ASETS_H
#define ASETS_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ASETS_ABI_VERSION 1

#if defined(_WIN32)
#define ASETS_API __declspec(dllexport)
#else
#define ASETS_API __attribute__((visibility("default")))
#endif

typedef enum asets_status {
    ASETS_OK = 0,
    ASETS_ERR_INVALID_ARG = 1,  /* bad sizes/pars/pointers */
    ASETS_ERR_ALPHA = 2,        /* "alpha(x) must be positive. Exiting..." */
    ASETS_ERR_CUDA = 3,         /* a CUDA runtime call failed */
    ASETS_ERR_OUT_OF_MEMORY = 4,
    ASETS_ERR_TIMEOUT = 5,      /* a bounded device-side wait ran out */
    ASETS_ERR_NO_DEVICE = 6,    /* no usable sm_103 GPU */
    ASETS_ERR_UNSUPPORTED = 7
} asets_status;

typedef enum asets_model {
    ASETS_BINARY = 0,
    ASETS_POTTS = 1,
    ASETS_ISHIKAWA = 2
} asets_model;

/* Where a pointer lives. */
typedef enum asets_memory { ASETS_HOST = 0, ASETS_DEVICE = 1 } asets_memory;

/* Solve options; pass NULL for the defaults. */
typedef struct asets_options {
    int flags;       /* ASETS_FLAG_* */
    int tile_config; /* 0 = default; k >= 1 selects the k-th tile variant of the kernel */
    int reserved[6];
} asets_options;

/* Form |p(x)| in double precision exactly as projStep does
 * (maxflow/asetsBinaryMF3D_mex.c:321-324), making u bit-identical to the
 * reference C.  Without it |p(x)| is formed in float (default, faster). */
#define ASETS_FLAG_EXACT 0x1
/* Skip the alpha(x) > 0 validation pass. */
#define ASETS_FLAG_NO_ALPHA_CHECK 0x2
/* Time the kernel variants (tile shapes, ring depths) on the problem -- one
 * chunk of iterations each, from the same initial state -- before solving
 * and use the fastest; the choice is cached per process (single solves by
 * model, size and exactness; batches by group and problem mix).  Ignored
 * when opt->tile_config selects a variant. */
#define ASETS_FLAG_AUTOTUNE 0x4

ASETS_API int asets_abi_version(void);
ASETS_API const char *asets_status_string(asets_status s);
/* Message of the last failure on the calling thread ("" if none). */
ASETS_API const char *asets_last_error(void);

/* ------------------------------------------------------------------------
 * Contexts.  A context owns a CUDA stream on one device, the device buffers
 * of the last problem shape (reused across calls of the same shape) and a
 * pinned staging area.  Calls on one context are serialised internally;
 * different contexts may be used from different threads.
 * ---------------------------------------------------------------------- */
typedef struct asets_context asets_context;

ASETS_API asets_status asets_context_create(int device, asets_context **out);
ASETS_API void asets_context_destroy(asets_context *ctx);
/* The process-wide context used by the mex entry points (device from
 * $ASETS_DEVICE, default 0), created on first use. */
ASETS_API asets_status asets_default_context(asets_context **out);
/* Launch on this CUDA stream (a cudaStream_t passed as void*, or NULL for the
 * context's own stream). */
ASETS_API asets_status asets_context_set_stream(asets_context *ctx, void *stream);
/* Failure-detection self-check (no counterpart in the reference): runs one
 * kernel whose bounded device-side wait (the kind every solver kernel uses on
 * its TMA and tensor-core completions) waits on a barrier that nothing
 * completes.  Expected result: ASETS_ERR_TIMEOUT after about one second, with
 * the context still usable. */
ASETS_API asets_status asets_selftest_wait_timeout(asets_context *ctx);

/* ------------------------------------------------------------------------
 * One-shot solvers with host pointers: the runMaxFlow() of each mex file,
 * same argument meaning and order (alpha, costs, sizes, maxIt, errBound, cc,
 * steps, outputs).  u/cvg/itNum follow the reference exactly:
 *   u      final labelling (binary N, Potts N*L, Ishikawa N*(L-1))
 *   cvg    maxIt entries, erriter per iteration, zero after the break
 *   itNum  index of the iteration that met errBound, or maxIt
 * seconds (optional, may be NULL) receives the wall time of the call.
 * ---------------------------------------------------------------------- */

/* replaces runMaxFlow, maxflow/asetsBinaryMF2D_mex.c:132-194 */
ASETS_API asets_status asets_binary_mf2d(asets_context *ctx, const asets_options *opt,
                                         const float *alpha, const float *Cs, const float *Ct,
                                         int Nx, int Ny, int maxIt, float errBound, float cc,
                                         float steps, float *u, float *cvg, int *itNum,
                                         float *seconds);
/* replaces runMaxFlow, maxflow/asetsBinaryMF3D_mex.c:137-203 */
ASETS_API asets_status asets_binary_mf3d(asets_context *ctx, const asets_options *opt,
                                         const float *alpha, const float *Cs, const float *Ct,
                                         int Nx, int Ny, int Nz, int maxIt, float errBound,
                                         float cc, float steps, float *u, float *cvg, int *itNum,
                                         float *seconds);
/* replaces runMaxFlow, maxflow/asetsPotts2D_mex.c:138-210 */
ASETS_API asets_status asets_potts2d(asets_context *ctx, const asets_options *opt,
                                     const float *alpha, const float *Ct, int Nx, int Ny,
                                     int nLab, int maxIt, float errBound, float cc, float steps,
                                     float *u, float *cvg, int *itNum, float *seconds);
/* replaces runMaxFlow, maxflow/asetsPotts3D_mex.c:144-217 */
ASETS_API asets_status asets_potts3d(asets_context *ctx, const asets_options *opt,
                                     const float *alpha, const float *Ct, int Nx, int Ny, int Nz,
                                     int nLab, int maxIt, float errBound, float cc, float steps,
                                     float *u, float *cvg, int *itNum, float *seconds);
/* replaces runMaxFlow, maxflow/asetsIshikawa2D_mex.c:136-219 */
ASETS_API asets_status asets_ishikawa2d(asets_context *ctx, const asets_options *opt,
                                        const float *alpha, const float *Ct, int Nx, int Ny,
                                        int nLab, int maxIt, float errBound, float cc,
                                        float steps, float *u, float *cvg, int *itNum,
                                        float *seconds);
/* replaces runMaxFlow, maxflow/asetsIshikawa3D_mex.c:141-228 */
ASETS_API asets_status asets_ishikawa3d(asets_context *ctx, const asets_options *opt,
                                        const float *alpha, const float *Ct, int Nx, int Ny,
                                        int Nz, int nLab, int maxIt, float errBound, float cc,
                                        float steps, float *u, float *cvg, int *itNum,
                                        float *seconds);

/* ------------------------------------------------------------------------
 * Solver objects: device-resident problems.  Inputs are uploaded once
 * (host or device pointers, Matlab layout); run() iterates on the device;
 * results are read back on demand.  This is the path for repeated solves,
 * for device-resident pipelines, and for warm starts.
 * ---------------------------------------------------------------------- */
typedef struct asets_solver asets_solver;

/* dims: Ny (rows), Nx (cols), Nz (slices, 1 for 2D); dim is 2 or 3;
 * nLab is 1 for binary. */
ASETS_API asets_status asets_solver_create(asets_context *ctx, asets_model model, int dim,
                                           int Ny, int Nx, int Nz, int nLab,
                                           asets_solver **out);
ASETS_API void asets_solver_destroy(asets_solver *s);
/* Cs is used by the binary model only (NULL otherwise).  alpha has 1 (binary),
 * L (Potts) or L-1 (Ishikawa) slices. */
ASETS_API asets_status asets_solver_set_inputs(asets_solver *s, asets_memory where,
                                               const float *Cs, const float *Ct,
                                               const float *alpha);
/* Copy the current inputs out (any pointer may be NULL); on a coarse level
 * of a multilevel chain these are the restricted inputs. */
ASETS_API asets_status asets_solver_get_inputs(asets_solver *s, asets_memory where, float *Cs,
                                               float *Ct, float *alpha);
/* Warm start: initial u/ps/pt instead of the reference's init (the flows
 * still start at zero, as calloc'd in runMaxFlow).  Shapes: binary u,ps,pt N;
 * Potts u N*L, ps N, pt N*L; Ishikawa u N*(L-1), pt N*L (ps NULL).  Pass all
 * NULL to return to the cold start. */
ASETS_API asets_status asets_solver_set_initial(asets_solver *s, asets_memory where,
                                                const float *u0, const float *ps0,
                                                const float *pt0);
/* Spatial flows: initial values and the state after a run (no counterpart in
 * the reference, whose runMaxFlow keeps bx/by/bz internal and starts them at
 * zero).  Layout as the reference's arrays: flow_labels*N floats each
 * (1 binary, L Potts, L-1 Ishikawa), bx(y,x[,z]) the flow across the face
 * between x-1 and x, by between y-1 and y, bz between z-1 and z (3D only;
 * pass NULL in 2D).  Border faces (index 0 of their axis) are taken as zero.
 * Initial flows apply to every later run until cleared with all NULL or by
 * asets_solver_set_initial(all NULL).  Together with set_initial and
 * get_u/get_flows this saves and restores the full iteration state. */
ASETS_API asets_status asets_solver_set_initial_flows(asets_solver *s, asets_memory where,
                                                      const float *bx, const float *by,
                                                      const float *bz);
ASETS_API asets_status asets_solver_get_spatial_flows(asets_solver *s, asets_memory where,
                                                      float *bx, float *by, float *bz);
/* Run up to maxIt iterations; itNum as in the one-shot calls. */
ASETS_API asets_status asets_solver_run(asets_solver *s, const asets_options *opt, int maxIt,
                                        float errBound, float cc, float steps, int *itNum);
ASETS_API asets_status asets_solver_get_u(asets_solver *s, asets_memory where, float *u);
/* n = number of entries to copy (<= maxIt of the last run). */
ASETS_API asets_status asets_solver_get_cvg(asets_solver *s, asets_memory where, float *cvg,
                                            int n);
/* Final source/sink flows (ps: binary/Potts N, NULL allowed; pt: binary N,
 * Potts/Ishikawa N*L). */
ASETS_API asets_status asets_solver_get_flows(asets_solver *s, asets_memory where, float *ps,
                                              float *pt);
/* Multilevel (coarse-to-fine) solve (no counterpart in the reference): the
 * problem is restricted to grids with half the cells per axis (cost terms
 * 2*mean over each 2x2(x2) block, alpha the block mean), the coarsest grid is
 * solved first, and each solved state (u, ps, pt and the flows) is prolonged
 * to the next finer grid as its initial state (u copied, ps/pt halved, flows
 * interpolated along their axis), down to the original grid, whose run gives
 * u, erriter and itNum as asets_solver_run does.  Every level runs with the
 * same maxIt, errBound, cc and steps.  Coarsening stops when an axis would
 * fall below 4 cells (at most 8 levels).  The coarse levels are solvers
 * owned by `s`; an initial state set on the coarsest level (through
 * asets_solver_level) is used by its run, one set on `s` itself is replaced
 * by the prolonged state.  levels = 1 is asets_solver_run. */
ASETS_API asets_status asets_solver_run_multilevel(asets_solver *s, const asets_options *opt,
                                                   int levels, int maxIt, float errBound,
                                                   float cc, float steps, int *itNum);
/* Create the coarse levels and restrict the current inputs to them without
 * solving; *levels_out = the number of levels the grid allows (<= levels). */
ASETS_API asets_status asets_solver_multilevel_prepare(asets_solver *s, int levels,
                                                       int *levels_out);
/* Level `level` (0 = s) of the multilevel chain; owned by s (do not destroy). */
ASETS_API asets_status asets_solver_level(asets_solver *s, int level, asets_solver **out);
/* Per-level itNum and device ms of the last multilevel run (level 0 = s). */
ASETS_API asets_status asets_solver_multilevel_stats(asets_solver *s, int cap, int *iters,
                                                     float *ms, int *levels_out);
/* Device time (ms) of the last run's iteration loop, from CUDA events on the
 * launch stream, and the number of kernel launches it made. */
ASETS_API asets_status asets_solver_last_run_stats(asets_solver *s, float *ms,
                                                   int *kernel_launches);

/* ------------------------------------------------------------------------
 * Batches: many independent binary problems (2D and 3D, any sizes) solved
 * together.  Each iteration is one persistent launch per dimension over the
 * work items of all problems that have not converged; every problem keeps
 * the reference's own stopping rule, erriter and itNum, exactly as if solved
 * alone.  Iteration chunks run as CUDA graphs.  No counterpart in the
 * reference (which solves one problem per call).
 * ---------------------------------------------------------------------- */
typedef struct asets_batch asets_batch;

ASETS_API asets_status asets_batch_create(asets_context *ctx, asets_batch **out);
ASETS_API void asets_batch_destroy(asets_batch *b);
/* Add a solver whose inputs are set (any model, 2D or 3D); the batch does
 * not own it.  Members are grouped by dimension and by binary / labelled
 * model; a group shares one fused-pass launch per iteration, and each
 * labelled member's label kernel follows it. */
ASETS_API asets_status asets_batch_add(asets_batch *b, asets_solver *s);
/* Solve every member; itNums (optional) receives one itNum per member in
 * the order they were added.  Results are read from each solver
 * (asets_solver_get_u / _get_cvg). */
ASETS_API asets_status asets_batch_run(asets_batch *b, const asets_options *opt, int maxIt,
                                       float errBound, float cc, float steps, int *itNums);
/* Device time of the last run, kernel launches, iterations summed over the
 * members, and the tile configuration used for the binary 2D and 3D groups. */
ASETS_API asets_status asets_batch_last_run_stats(asets_batch *b, float *ms, int *kernel_launches,
                                                  int *iterations, int *tile_configs);
/* Coarse-to-fine solve of every member, the batch form of
 * asets_solver_run_multilevel: level k of all members that have one runs as
 * one batch (coarsest first, each member's coarsest level from its own
 * initial state, e.g. a learned warm start set on asets_solver_level()),
 * every finer level from the prolonged solution of the level below.
 * itNums receives the full-resolution itNum per member; per-level itNums
 * and the device time of each level's batch are in
 * asets_solver_multilevel_stats of each member. */
ASETS_API asets_status asets_batch_run_multilevel(asets_batch *b, const asets_options *opt,
                                                  int levels, int maxIt, float errBound,
                                                  float cc, float steps, int *itNums);

/* ------------------------------------------------------------------------
 * Learned warm start building block (no counterpart in the reference):
 * one 3x3x3 convolution with 16 input and 16 output channels on the tensor
 * cores, BF16 operands and FP32 accumulation, zero padding at the volume
 * border.  x: device BF16 [Nz][Nx][Ny][16] (16-byte aligned); w: device BF16
 * [27][16 in][16 out], tap = (dz*3 + dx)*3 + dy for offsets dz,dx,dy in
 * -1..1; bias: device float[16] or NULL; mask: device BF16 like x or NULL
 * (output channel c of voxel v kept only where mask[v][c] > 0); y: device
 * BF16 or (out_fp32) float [..][16].  relu applies max(0, .).  With flip the
 * transposed convolution is computed (taps mirrored, w[t] transposed): the
 * gradient with respect to the input.
 * ---------------------------------------------------------------------- */
ASETS_API asets_status asets_conv3d_bf16(asets_context *ctx, const void *x, const void *w,
                                         const float *bias, const void *mask, void *y, int Ny,
                                         int Nx, int Nz, int relu, int out_fp32, int flip);

/* ------------------------------------------------------------------------
 * Learned warm start for the Potts model (no counterpart in the reference):
 * a network of four 3x3x3 convolutional layers with 16 hidden channels and
 * ReLU maps (Ct_1..Ct_L, alpha) to an initial state for
 * asets_solver_set_initial / asets_solver_set_initial_flows: u_1..u_L, ps,
 * pt_1..pt_L and the spatial flows bx, by, bz (L slices each).  Forward and
 * data-gradient convolutions run on the tensor cores (BF16, FP32
 * accumulation), weight gradients in FP32; training is Adam on an MSE loss
 * against solver states (flows relative to alpha).  All arrays are device
 * pointers in Matlab layout (label slowest); alpha is one slice.
 * Parameters: 5 blocks x (27*16*16 weights [tap][in][out] + 16 biases),
 * float; blocks 0-2 are the hidden layers, blocks 3 and 4 the two 16-channel
 * halves of the 32-channel output layer.
 * ---------------------------------------------------------------------- */
typedef struct asets_wsnet asets_wsnet;

ASETS_API int asets_wsnet_num_params(void);
/* 1 <= nLab <= 6; weights He-initialised from `seed`. */
ASETS_API asets_status asets_wsnet_create(asets_context *ctx, int nLab, unsigned long long seed,
                                          asets_wsnet **out);
ASETS_API void asets_wsnet_destroy(asets_wsnet *n);
ASETS_API asets_status asets_wsnet_get_params(asets_wsnet *n, float *host_params);
ASETS_API asets_status asets_wsnet_set_params(asets_wsnet *n, const float *host_params);
/* u0 (N*L, clamped to [0,1]), ps0 (N), pt0 (N*L) and optionally the flows
 * bx0, by0, bz0 (N*L each; all three or none) for a Ny x Nx x Nz volume. */
ASETS_API asets_status asets_wsnet_predict(asets_wsnet *n, int Ny, int Nx, int Nz,
                                           const float *Ct, const float *alpha, float *u0,
                                           float *ps0, float *pt0, float *bx0, float *by0,
                                           float *bz0);
/* Loss and parameter gradients (host) against a solver state. */
ASETS_API asets_status asets_wsnet_gradients(asets_wsnet *n, int Ny, int Nx, int Nz,
                                             const float *Ct, const float *alpha, const float *u,
                                             const float *ps, const float *pt, const float *bx,
                                             const float *by, const float *bz, float *host_grads,
                                             float *loss);
/* One Adam step (learning rate lr) on one solved volume; returns the loss. */
ASETS_API asets_status asets_wsnet_train_step(asets_wsnet *n, int Ny, int Nx, int Nz,
                                              const float *Ct, const float *alpha,
                                              const float *u, const float *ps, const float *pt,
                                              const float *bx, const float *by, const float *bz,
                                              float lr, float *loss);

/* ------------------------------------------------------------------------
 * Star-shape Potts 2D (maxflow/asetsPotts2D_starShape.m, a Matlab solver:
 * no counterpart in the reference's C code).  Same arguments as the .m
 * function, computed in double precision as Matlab does: Ct, alpha
 * rows x cols x nlab (host, Matlab layout); init_points nlab x 2 of 1-based
 * (column, row) seed points (ss_initPoints); pars = [rows, cols, nlab,
 * iterNum, beta, cc, steps, stepv].  Outputs u (rows*cols*nlab), erriter
 * (iterNum, zero after the break), itNum = the 1-based iteration of the
 * break (erriter < beta) or iterNum, seconds = wall time.
 * ---------------------------------------------------------------------- */
ASETS_API asets_status asets_potts2d_starshape(asets_context *ctx, const double *Ct,
                                               const double *alpha, int rows, int cols,
                                               int nlab, int iterNum, double beta, double cc,
                                               double steps, double stepv,
                                               const int *init_points, double *u,
                                               double *erriter, int *itNum, float *seconds);

/* ------------------------------------------------------------------------
 * Hierarchical max-flow, full-flow iteration (maxflow/asetsHMF2D.m and
 * asetsHMF3D.m, MaxFullFlow; Matlab classes with no counterpart in the
 * reference's C code).  precision 4 (float) or 8 (double), as the class of
 * the cost terms.  The tree: num_nodes nodes in pre-order, parent[0] = -1
 * (the root), parent[i] < i, children of a node in index order.  Ct[i]:
 * D1*D2*D3 costs of leaf i (Matlab layout; NULL for inner nodes);
 * alpha_arrays[i] a per-pixel alpha or NULL, then alpha_scalars[i] is used.
 * Runs numIts iterations (UpdateSinkFlows, UpdateLabels,
 * UpdateSpatialFlows; isotropic flows only) and copies out any non-NULL
 * per-node result: u, pt, div, g (D1*D2*D3), the spatial flows p1
 * ((D1-1)*D2*D3, the class's px), p2 (D1*(D2-1)*D3, py), p3
 * (D1*D2*(D3-1), pz, 3D only), and CalculateCostsFullFlow's dataCost and
 * reguCost per node (each including its subtree).  All host memory.
 * ---------------------------------------------------------------------- */
ASETS_API asets_status asets_hmf_full_flow(asets_context *ctx, int precision, int dim, int D1,
                                           int D2, int D3, int num_nodes, const int *parent,
                                           const void *const *Ct,
                                           const void *const *alpha_arrays,
                                           const double *alpha_scalars, int numIts,
                                           double steps, double cc, void *const *u,
                                           void *const *pt, void *const *div, void *const *g,
                                           void *const *p1, void *const *p2, void *const *p3,
                                           double *data_cost, double *regu_cost);

/* HMF with the class's optional parts (maxflow/asetsHMF2D.m, asetsHMF3D.m):
 * algorithm ASETS_HMF_FULL_FLOW (MaxFullFlow, as asets_hmf_full_flow) or
 * ASETS_HMF_PSEUDO_FLOW (MaxPseudoFlow: reads every leaf's initial labels
 * from u[i] and writes the labels back, an inner node's u being the sum of
 * its children's; pt is not touched and no costs are formed, as in the
 * class).  lx, ly, lz: per node a direction field (D1*D2*D3, the class's
 * geodesic shape constraint) or null; a node with lx needs ly (and lz in
 * 3D).  The fields are normalised to unit length at initialisation (0 where
 * the length is at most 0.001) and the normalised fields are written back
 * into the same arrays, as the class keeps them.  Other arguments as
 * asets_hmf_full_flow. */
typedef enum { ASETS_HMF_FULL_FLOW = 0, ASETS_HMF_PSEUDO_FLOW = 1 } asets_hmf_algorithm;
ASETS_API asets_status asets_hmf_run(asets_context *ctx, int algorithm, int precision, int dim,
                                     int D1, int D2, int D3, int num_nodes, const int *parent,
                                     const void *const *Ct, const void *const *alpha_arrays,
                                     const double *alpha_scalars, void *const *lx,
                                     void *const *ly, void *const *lz, int numIts, double steps,
                                     double cc, void *const *u, void *const *pt,
                                     void *const *div, void *const *g, void *const *p1,
                                     void *const *p2, void *const *p3, double *data_cost,
                                     double *regu_cost);

/* DAG max-flow, full-flow iteration (maxflow/asetsDAGMF2D.m and
 * asetsDAGMF3D.m, MaxFullFlow; Matlab classes with no counterpart in the
 * reference's C code): as asets_hmf_full_flow, but a node may have several
 * parents.  The graph: node 0 is the root; nchild[i] children of node i,
 * listed in order in the flattened `children` (inner nodes need two or
 * more, as the reference's initialisation does).  Each child is weighted
 * 1/(its number of parents); nodes are visited in the class's own top-down
 * list (depth-first, a node once all its parents are listed).  Outputs as
 * asets_hmf_full_flow plus pn (the flow pushed down to nodes with several
 * parents); no costs. */
ASETS_API asets_status asets_dag_full_flow(asets_context *ctx, int precision, int dim, int D1,
                                           int D2, int D3, int num_nodes, const int *nchild,
                                           const int *children, const void *const *Ct,
                                           const void *const *alpha_arrays,
                                           const double *alpha_scalars, int numIts,
                                           double steps, double cc, void *const *u,
                                           void *const *pt, void *const *pn, void *const *div,
                                           void *const *g, void *const *p1, void *const *p2,
                                           void *const *p3);

/* DAG max-flow with direction fields (asetsDAGMF2D.m / 3D lx, ly, lz):
 * as asets_dag_full_flow, the fields as in asets_hmf_run. */
ASETS_API asets_status asets_dag_run(asets_context *ctx, int precision, int dim, int D1, int D2,
                                     int D3, int num_nodes, const int *nchild,
                                     const int *children, const void *const *Ct,
                                     const void *const *alpha_arrays,
                                     const double *alpha_scalars, void *const *lx,
                                     void *const *ly, void *const *lz, int numIts, double steps,
                                     double cc, void *const *u, void *const *pt,
                                     void *const *pn, void *const *div, void *const *g,
                                     void *const *p1, void *const *p2, void *const *p3);

/* ------------------------------------------------------------------------
 * Matlab-semantics solvers: the reference's Matlab twins of the six solvers
 * (maxflow/asets{BinaryMF,Potts,Ishikawa}{2D,3D}.m, the path its tutorials
 * run with gpuArray), computed in the class of Ct (precision 4 or 8) with
 * the .m files' initialisation, expression order and `<` break rule.
 * model: 0 binary (Cs needed), 1 Potts, 2 Ishikawa; Ct rows*cols*slices*L
 * (binary L = 1); alpha per flow label (binary 1, Potts L, Ishikawa L-1
 * slices); host arrays of that precision.  Outputs u (binary N, Potts N*L,
 * Ishikawa N*(L-1)), erriter (iterNum, zero after the break; Ishikawa's
 * denominator is N*L-1 as in the .m files), itNum = the 1-based iteration
 * of the break or iterNum, seconds = wall time.
 * ---------------------------------------------------------------------- */
ASETS_API asets_status asets_matlab_solve(asets_context *ctx, int model, int precision, int dim,
                                          int rows, int cols, int slices, int nlab,
                                          const void *Cs, const void *Ct, const void *alpha,
                                          int iterNum, double beta, double cc, double steps,
                                          void *u, void *erriter, int *itNum, float *seconds);

/* ------------------------------------------------------------------------
 * Cost terms and regularisation weights on the GPU: the step before the
 * solvers in the reference's applications (the applications folder; no counterpart
 * in its C code).  Arrays in Matlab layout, label slowest; `where` says
 * whether the pointers are host or device memory.  Normalisation divides by
 * the volume's own range, (I - min I) / (max I - min I), in float32.
 * ---------------------------------------------------------------------- */
/* L1 intensity cost (L1IntensitySegmentation2D.m:32-45): Ct_l = |I' - m_l|,
 * I' the normalised image (normalize != 0) or I itself; 1 <= L <= 32. */
ASETS_API asets_status asets_cost_l1(asets_context *ctx, asets_memory where, const float *img,
                                     long long n, const float *models, int L, int normalize,
                                     float *Ct);
/* -log probability cost (atlasProbabilityMapsRegularization3D.m:45-53):
 * Ct = -log(p + eps) for N*L probabilities. */
ASETS_API asets_status asets_cost_neglog(asets_context *ctx, asets_memory where,
                                         const float *prob, long long n, int L, float eps,
                                         float *Ct);
/* Histogram log-likelihood cost (interactiveGraphCutSegmentation3D.m:104-122):
 * x = I' * 255; for each label l = 1..L the 256-bin histogram of x over the
 * voxels with scribbles == l (bin k holds k <= x < k+1, the last also
 * x == 255, as histc on 0:255), normalised to probabilities P_l; then
 * Ct_l = -log10(P_l[round(x)] + eps) (round half away from zero, as
 * uint16()).  hist_out (host, L*256, may be NULL) receives the counts. */
ASETS_API asets_status asets_cost_histogram_ll(asets_context *ctx, asets_memory where,
                                               const float *img, const int *scribbles,
                                               long long n, int L, double eps, float *Ct,
                                               unsigned int *hist_out);
/* Contrast-sensitive regularisation weight (smoothManualSegmentations2D.m:82-91;
 * the binary 3D workload's alpha): alpha = a + b*exp(-c*|grad I'|^p), p = 2
 * if squared else 1, gradient as Matlab's gradient (central differences
 * inside, one-sided at the border, 2D when Nz == 1), replicated over L
 * slices. */
ASETS_API asets_status asets_alpha_contrast(asets_context *ctx, asets_memory where,
                                            const float *img, int Ny, int Nx, int Nz,
                                            int normalize, float a, float b, float c, int squared,
                                            int L, float *alpha);

/* ------------------------------------------------------------------------
 * Allocation-free binary 3D solve.  No counterpart in the reference: it
 * exists for callers that cannot allocate device memory while they run -- a
 * host whose GPU memory is owned by another allocator (a framework's caching
 * allocator that has reserved the device, Matlab's gpuArray memory manager
 * around a mex file) or a pipeline that reserves everything at start-up and
 * forbids allocation afterwards.
 *
 * Same solve as asets_binary_mf3d(), but alpha/Cs/Ct/u/cvg are DEVICE
 * pointers (Matlab layout; cvg has maxIt entries), itNum is a host pointer,
 * and stream is a cudaStream_t (NULL: the default stream) on the current
 * device.  It calls no cudaMalloc/cudaFree or other allocating routine: its
 * scratch lives in one fixed device array of about 15 MiB, device memory of
 * the library's module.  Under CUDA's default lazy module loading that array
 * is reserved by the first call on a device (which looks up its address),
 * or at library load with CUDA_MODULE_LOADING=EAGER, and held until the
 * process exits: a caller that later hands the GPU to another allocator
 * makes one small call first (a 1x1x1 problem with maxIt 0), before that
 * allocator reserves the device and before any stream capture.  If the
 * first call cannot reserve it, it returns ASETS_ERR_OUT_OF_MEMORY.
 * Problems whose padded volume (row pitch x Nx x Nz, the pitch being Ny
 * rounded up to a multiple of 32, or of 4 below 32 rows) exceeds 262144
 * voxels are rejected with ASETS_ERR_INVALID_ARG.  All calls on a device
 * share the array and keep the previous call's contents (the solve clears
 * what must start at zero); calls are serialised inside the library and each
 * waits for its GPU work before returning, on success and on error -- two
 * calls whose GPU work overlapped would race on the shared scratch.
 * ---------------------------------------------------------------------- */
ASETS_API asets_status asets_binary_mf3d_noalloc(const asets_options *opt, const float *alpha,
                                                 const float *Cs, const float *Ct, int Nx,
                                                 int Ny, int Nz, int maxIt, float errBound,
                                                 float cc, float steps, float *u, float *cvg,
                                                 int *itNum, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ASETS_H */
