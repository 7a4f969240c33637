// Host runtime of libasetscuda: contexts, device-resident solver objects,
// TMA descriptors, the iteration driver and the C ABI of include/asets.h.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "asets.h"
#include "internal.h"

// NVTX range for profilers (a no-op unless a tool is attached): solves,
// batches, multilevel levels, autotuning and each CUDA-graph iteration chunk
// show up on the timeline under these names.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

using namespace asets;

// ---------------------------------------------------------------- errors
static thread_local std::string g_last_error;

static asets_status fail(asets_status s, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return s;
}

namespace asets {
void set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }
}  // namespace asets

static asets_status cuda_fail(cudaError_t e, const char *what)
{
    asets_status s = (e == cudaErrorMemoryAllocation) ? ASETS_ERR_OUT_OF_MEMORY : ASETS_ERR_CUDA;
    cudaGetLastError();  // clear a non-sticky error
    return fail(s, "%s: %s", what, cudaGetErrorString(e));
}

#define CU_TRY(call)                                 \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess)                       \
            return cuda_fail(e_, #call);             \
    } while (0)

// RAII: make ctx->device current for the duration of an API call.
struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess)
            prev = -1;
        ok = (prev == dev) || (cudaSetDevice(dev) == cudaSuccess);
    }
    ~DeviceGuard()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev)
            cudaSetDevice(prev);
    }
};

// ---------------------------------------------------------------- context

struct asets_context {
    int device = 0;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    EncodeTiledFn encode = nullptr;
    std::recursive_mutex mu;
    asets_solver *cached = nullptr;  // solver reused by the one-shot calls
    int *pinned_flags = nullptr;     // host-visible done flags of in-flight chunks
    cudaMemPool_t pool = nullptr;    // scratch of the cost-term calls (keeps small blocks mapped)
};

struct ChunkGraph {
    cudaGraphExec_t exec = nullptr;
    const void *key_fn = nullptr;
    float key_cc = 0.f;
    const void *key_cvg = nullptr;
    void reset()
    {
        if (exec)
            cudaGraphExecDestroy(exec);
        exec = nullptr;
        key_fn = nullptr;
    }
};

struct asets_solver {
    asets_context *ctx = nullptr;
    asets_model model = ASETS_BINARY;
    int dim = 3, ny = 0, nx = 0, nz = 0, nlab = 1;
    // kernel view: rows, columns (1 in 2D), stream axis
    int nr = 0, nc = 0, ns = 0;
    long long pitch = 0, plane = 0, cells = 0;  // cells = padded cells per label
    int flow_labels = 1, alpha_labels = 1, ct_labels = 1, pt_labels = 1, u_labels = 1;
    // device buffers (padded layout)
    std::vector<void *> allocations;
    float *cs = nullptr, *ct = nullptr, *alpha = nullptr;
    float *b[2][3] = {};
    float *ps[2] = {}, *pt[2] = {}, *u[2] = {};
    float *dv = nullptr;
    float *warm_u = nullptr, *warm_ps = nullptr, *warm_pt = nullptr;
    bool warm = false;
    float *warm_b[3] = {nullptr, nullptr, nullptr};  // initial spatial flows (padded)
    bool warm_flows = false;
    bool inputs_set = false;
    bool alpha_ok = true;
    IterControl *ctl = nullptr;
    double *partials = nullptr;
    int partials_cap = 0;
    float *cvg = nullptr;
    int cvg_cap = 0;
    // results of the last run
    int last_max_it = 0;
    int final_parity = 0;
    int flow_parity = 0;  // b[flow_parity] holds the flows after the last run
    // multilevel solve: the next coarser level (owned) and per-level results
    asets_solver *coarse = nullptr;
    int ml_levels = 0;
    int ml_iters[kMaxLevels] = {};
    float ml_ms[kMaxLevels] = {};
    float last_ms = 0.f;
    int last_launches = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t flag_ev[2] = {nullptr, nullptr};
    // kernel setup cache: this problem as a batch of one
    const StencilVariant *variant = nullptr;
    int grid = 0;
    ProblemDesc desc;                  // host copy, uploaded at each run
    ProblemDesc *d_desc = nullptr;
    ProblemDesc *d_desc_replay = nullptr;  // one-iteration re-run after a two-iteration pass
    int *d_item_problem = nullptr;
    double *d_item_partials = nullptr;
    unsigned int *d_queue = nullptr;
    int items_cap = 0;
    BatchArgs bargs;
    ChunkGraph graph;
    int last_iters = 0;  // iterations executed by the last run
};

static asets_status get_encoder(asets_context *ctx)
{
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                     cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
        return fail(ASETS_ERR_CUDA, "cuTensorMapEncodeTiled unavailable from the driver");
    ctx->encode = reinterpret_cast<EncodeTiledFn>(fn);
    return ASETS_OK;
}

namespace asets {
EncodeTiledFn context_encoder(asets_context *ctx) { return ctx->encode; }
int context_num_sms(asets_context *ctx) { return ctx->num_sms; }
int context_device(asets_context *ctx) { return ctx->device; }
cudaStream_t context_stream(asets_context *ctx) { return ctx->stream; }

cudaMemPool_t context_pool(asets_context *ctx)
{
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    if (!ctx->pool) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = ctx->device;
        if (cudaMemPoolCreate(&ctx->pool, &props) != cudaSuccess) {
            cudaGetLastError();
            ctx->pool = nullptr;
            return nullptr;
        }
        // blocks up to this size stay mapped between calls; larger frees
        // go back to the device at the next synchronisation
        cuuint64_t keep = 64ull << 20;
        cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    return ctx->pool;
}
}  // namespace asets

extern "C" ASETS_API int asets_abi_version(void) { return ASETS_ABI_VERSION; }

extern "C" ASETS_API const char *asets_status_string(asets_status s)
{
    switch (s) {
    case ASETS_OK: return "ok";
    case ASETS_ERR_INVALID_ARG: return "invalid argument";
    case ASETS_ERR_ALPHA: return "alpha(x) must be positive. Exiting...";
    case ASETS_ERR_CUDA: return "CUDA error";
    case ASETS_ERR_OUT_OF_MEMORY: return "out of device memory";
    case ASETS_ERR_TIMEOUT: return "device wait timed out";
    case ASETS_ERR_NO_DEVICE: return "no usable sm_103 GPU";
    case ASETS_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

extern "C" ASETS_API const char *asets_last_error(void) { return g_last_error.c_str(); }

extern "C" ASETS_API asets_status asets_context_create(int device, asets_context **out)
{
    if (!out)
        return fail(ASETS_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(ASETS_ERR_NO_DEVICE, "no CUDA device (%s)", cudaGetErrorString(e));
    }
    if (device < 0 || device >= n)
        return fail(ASETS_ERR_INVALID_ARG, "device %d out of range (0..%d)", device, n - 1);
    cudaDeviceProp prop;
    CU_TRY(cudaGetDeviceProperties(&prop, device));
    if (!(prop.major == 10 && prop.minor == 3))
        return fail(ASETS_ERR_NO_DEVICE, "device %d is sm_%d%d; libasetscuda is built for sm_103a",
                    device, prop.major, prop.minor);
    DeviceGuard guard(device);
    if (!guard.ok)
        return fail(ASETS_ERR_CUDA, "cudaSetDevice(%d) failed", device);
    std::unique_ptr<asets_context> ctx(new asets_context);
    ctx->device = device;
    ctx->num_sms = prop.multiProcessorCount;
    asets_status s = get_encoder(ctx.get());
    if (s != ASETS_OK)
        return s;
    CU_TRY(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
    ctx->stream = ctx->own_stream;
    CU_TRY(cudaMallocHost(&ctx->pinned_flags, 64 * sizeof(int)));
    *out = ctx.release();
    return ASETS_OK;
}

extern "C" ASETS_API void asets_solver_destroy(asets_solver *s);

extern "C" ASETS_API void asets_context_destroy(asets_context *ctx)
{
    if (!ctx)
        return;
    {
        DeviceGuard guard(ctx->device);
        if (ctx->cached)
            asets_solver_destroy(ctx->cached);
        if (ctx->own_stream) {
            cudaStreamSynchronize(ctx->own_stream);
            cudaStreamDestroy(ctx->own_stream);
        }
        if (ctx->pinned_flags)
            cudaFreeHost(ctx->pinned_flags);
        if (ctx->pool)
            cudaMemPoolDestroy(ctx->pool);  // every call freed its blocks before returning
    }
    delete ctx;
}

extern "C" ASETS_API asets_status asets_default_context(asets_context **out)
{
    static std::mutex mu;
    static asets_context *ctx = nullptr;
    static asets_status status = ASETS_OK;
    static bool tried = false;
    if (!out)
        return fail(ASETS_ERR_INVALID_ARG, "out is NULL");
    std::lock_guard<std::mutex> lock(mu);
    if (!tried || (!ctx && status != ASETS_ERR_NO_DEVICE)) {
        tried = true;
        const char *env = getenv("ASETS_DEVICE");
        int dev = env ? atoi(env) : 0;
        status = asets_context_create(dev, &ctx);
    }
    *out = ctx;
    if (!ctx)
        return status != ASETS_OK ? status : fail(ASETS_ERR_NO_DEVICE, "no default context");
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_selftest_wait_timeout(asets_context *ctx)
{
    if (!ctx)
        return fail(ASETS_ERR_INVALID_ARG, "ctx is NULL");
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    DeviceGuard guard(ctx->device);
    int *d_err = nullptr;
    CU_TRY(cudaMallocAsync(&d_err, sizeof(int), ctx->stream));
    int h_err = 0;
    cudaError_t e = cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream);
    if (e == cudaSuccess)
        e = launch_wait_selftest(d_err, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    cudaFreeAsync(d_err, ctx->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "wait self-test");
    if (h_err & DEV_ERR_TIMEOUT)
        return fail(ASETS_ERR_TIMEOUT, "a device-side wait timed out (self-test)");
    return fail(ASETS_ERR_CUDA, "the self-test wait did not time out");
}

extern "C" ASETS_API asets_status asets_context_set_stream(asets_context *ctx, void *stream)
{
    if (!ctx)
        return fail(ASETS_ERR_INVALID_ARG, "ctx is NULL");
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    return ASETS_OK;
}

// ---------------------------------------------------------------- solver
static asets_status dalloc(asets_solver *s, float **p, size_t floats)
{
    void *ptr = nullptr;
    cudaError_t e = cudaMalloc(&ptr, std::max<size_t>(floats, 1) * sizeof(float));
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaMalloc");
    s->allocations.push_back(ptr);
    *p = static_cast<float *>(ptr);
    return ASETS_OK;
}

extern "C" ASETS_API void asets_solver_destroy(asets_solver *s)
{
    if (!s)
        return;
    asets_solver_destroy(s->coarse);
    DeviceGuard guard(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    s->graph.reset();
    for (void *p : s->allocations)
        cudaFree(p);
    if (s->ev0)
        cudaEventDestroy(s->ev0);
    if (s->ev1)
        cudaEventDestroy(s->ev1);
    for (int i = 0; i < 2; ++i)
        if (s->flag_ev[i])
            cudaEventDestroy(s->flag_ev[i]);
    if (s->ctx->cached == s)
        s->ctx->cached = nullptr;
    delete s;
}

static long long round_pitch(int nr)
{
    if (nr >= 32)
        return ((long long)nr + 31) / 32 * 32;
    return ((long long)nr + 3) / 4 * 4;
}

// Whether the solver can run the one-pass multi-label 2D kernel: it needs
// the second parity of pt/u/ps, allocated for the label counts it covers.
static bool has_fused(const asets_solver *s)
{
    return s->dim == 2 && s->model != ASETS_BINARY && s->pt[1] != s->pt[0];
}

// The kernel variants open to a solve, in tile_config order (entry k-1 for
// tile_config k): the one-pass multi-label 2D kernel first where it applies
// (not in a batch, whose group shares one variant across label counts), then
// the kind's table.
static std::vector<const StencilVariant *> solver_candidates(const asets_solver *s, int exact,
                                                             bool single)
{
    std::vector<const StencilVariant *> c;
    if (single && has_fused(s))
        for (int w = 0; const StencilVariant *f = fused2d_variant((int)s->model, s->nlab, exact, w); ++w)
            c.push_back(f);
    int n = 0;
    const StencilVariant *tab = stencil_variants(s->dim, s->model == ASETS_BINARY ? EPI_BINARY : EPI_DIV,
                                                 exact, &n);
    // a batch launch serves many problems: no whole-solve cooperative kernels
    for (int i = 0; i < n; ++i)
        if (single || !tab[i].persistent)
            c.push_back(&tab[i]);
    return c;
}

// Dynamic shared memory of a launch of variant v for the solver's label counts.
static int launch_smem(const asets_solver *s, const StencilVariant *v)
{
    return v->smem_bytes + v->smem_per_fl * s->flow_labels + v->smem_per_l * s->nlab;
}

// The function attribute covers every label count (8 flow labels, 9
// labels), so that solvers of different label counts can share a variant.
static int attr_smem(const StencilVariant *v)
{
    return v->smem_bytes + v->smem_per_fl * 8 + v->smem_per_l * 9;
}

// Blocks of a whole-solve cooperative launch of variant v that can be
// resident at once (0: it does not fit on an SM).
static long long persistent_slots(const asets_solver *s, const StencilVariant *v)
{
    const int smem = launch_smem(s, v);
    if (cudaFuncSetAttribute(v->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, attr_smem(v)) !=
        cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v->fn, v->nt, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return (long long)per_sm * s->ctx->num_sms;
}

// Tiles of the solver's problem per resident block in a whole-solve launch
// of v (0: not launchable).
static double persistent_load(const asets_solver *s, const StencilVariant *v)
{
    const long long slots = persistent_slots(s, v);
    if (slots < 1)
        return 0.0;
    const long long tiles = (long long)((s->nr + v->tr - 1) / v->tr) * ((s->ns + v->s_tile - 1) / v->s_tile);
    return (double)tiles / (double)slots;
}

// Largest multi-label 2D image (pixels) the whole-solve tile kernel takes by default.
static constexpr long long kTileLabelsMaxPx = 1LL << 17;
// Most 32 x 32 tiles per resident block the binary whole-solve kernel takes
// by default: fast, every tile resident at once (beyond that the
// two-iteration sweep wins); EXACT, up to eight (about 1600^2 pixels: the
// EXACT sweep runs one iteration per pass)
static constexpr double kTileBinaryMaxLoad = 1.0, kTileBinaryMaxLoadExact = 8.0;

static const StencilVariant *pick_variant(const asets_solver *s, int exact, int tile_config,
                                          bool single)
{
    std::vector<const StencilVariant *> match = solver_candidates(s, exact, single);
    if (match.empty())
        return nullptr;
    if (tile_config > 0 && tile_config <= (int)match.size())
        return match[tile_config - 1];
    // the one-pass multi-label kernels lead the list: three sweeps (in-step
    // update, one label warp, two), then 16 x 16 tiles (one launch per
    // iteration, the whole solve in one).  By default they run where they
    // measured faster than the two-pass form on a GB300: the whole-solve
    // tiles on images of up to 2^17 pixels (two tiles per block at most);
    // the sweeps on two
    // million pixels and more (two label warps for up to three flow labels,
    // one above), and half a million with six flow labels or more (in-step)
    int n_fused = 0;
    while (n_fused < (int)match.size() && match[n_fused]->epi == EPI_FUSED)
        ++n_fused;
    if (n_fused == 5) {
        const long long px = (long long)s->nr * s->ns;
        const int fl = s->flow_labels;
        const double load = persistent_load(s, match[4]);
        if (px <= kTileLabelsMaxPx && load > 0.0 && load <= 2.0)
            return match[4];
        if (px >= 2000000)
            return match[fl <= 3 ? 2 : 1];
        if (px >= 500000 && fl >= 6)
            return match[0];
    }
    match.erase(match.begin(), match.begin() + n_fused);
    // small binary 2D images: the whole solve in one cooperative launch when
    // every tile can be resident (16 x 16 tiles up to 2^17 pixels, else
    // 32 x 32; EXACT also with up to eight 32 x 32 tiles per block),
    // measured faster than the sweeps there
    if (single && s->dim == 2 && s->model == ASETS_BINARY) {
        const long long px = (long long)s->nr * s->ns;
        for (int want : {16, 32}) {
            if (want == 16 && px > (1LL << 17))
                continue;
            for (auto *v : match)
                if (v->persistent && v->s_tile == want) {
                    const double load = persistent_load(s, v);
                    const double most = want == 16 ? 1.0
                                                   : (exact ? kTileBinaryMaxLoadExact : kTileBinaryMaxLoad);
                    if (load > 0.0 && load <= most)
                        return v;
                }
        }
    }
    for (size_t i = 0; i < match.size();)
        if (match[i]->persistent || match[i]->s_tile > 0)
            match.erase(match.begin() + i);  // square tiles: by tile_config or the autotuner
        else
            ++i;
    if (s->dim == 2 && s->nr <= 112) {
        // short columns: the narrow 2D variant wastes fewer rows
        for (auto *v : match)
            if (v->tr < 112)
                return v;
    }
    return match[0];
}

// The solver's buffers as the iteration kernel sees them (both parities);
// `fused`: for the one-pass multi-label kernel, whose pt/u/ps ping-pong like
// the flows.
static StencilProblem stencil_problem_of(const asets_solver *s, bool fused)
{
    const bool binary = (s->model == ASETS_BINARY);
    StencilProblem p;
    memset(&p, 0, sizeof p);
    p.nr = s->nr;
    p.nc = s->nc;
    p.ns = s->ns;
    p.pitch = s->pitch;
    p.plane = s->plane;
    p.cells = s->cells;
    p.flow_labels = s->flow_labels;
    for (int par = 0; par < 2; ++par) {
        for (int k = 0; k < 3; ++k)
            p.b[par][k] = s->b[par][k];
        if (binary) {
            p.src[par][0] = s->ps[par];
            p.src[par][1] = s->pt[par];
            p.src[par][2] = s->u[par];
            p.dst_s[par][0] = s->ps[par ^ 1];
            p.dst_s[par][1] = s->pt[par ^ 1];
            p.dst_s[par][2] = s->u[par ^ 1];
        } else if (fused) {
            const int q = par ^ 1;
            const bool potts = (s->model == ASETS_POTTS);
            p.src[par][0] = potts ? s->ps[par] : s->pt[par];
            p.src[par][1] = s->pt[par];
            p.src[par][2] = s->u[par];
            p.dst_s[par][0] = potts ? s->ps[q] : s->pt[q];
            p.dst_s[par][1] = potts ? s->pt[q] : nullptr;
            p.dst_s[par][2] = s->u[q];
        } else if (s->model == ASETS_POTTS) {
            p.src[par][0] = s->ps[0];
            p.src[par][1] = s->pt[0];
            p.src[par][2] = s->u[0];
            p.dst_s[par][0] = s->dv;
        } else {
            p.src[par][0] = s->pt[0];
            p.src[par][1] = s->pt[0];
            p.src[par][2] = s->u[0];
            p.dst_s[par][0] = s->dv;
        }
    }
    if (binary) {
        p.src_labels[0] = p.src_labels[1] = p.src_labels[2] = 1;
    } else if (s->model == ASETS_POTTS) {
        p.src_labels[0] = 1;
        p.src_labels[1] = p.src_labels[2] = s->nlab;
    } else {
        p.src_labels[0] = p.src_labels[1] = s->nlab;
        p.src_labels[2] = s->nlab - 1;
    }
    for (int slot = 0; slot < NUM_SLOTS; ++slot) {
        p.lab_mul[slot] = binary ? 0 : 1;
        p.lab_add[slot] = 0;
    }
    if (s->model == ASETS_POTTS)
        p.lab_mul[SL_S0] = 0;  // one shared source flow
    if (s->model == ASETS_ISHIKAWA)
        p.lab_add[SL_S1] = 1;  // pt_{k+1}
    p.alpha = s->alpha;
    p.alpha_labels = s->alpha_labels;
    p.cs = s->cs;
    p.ct = s->ct;
    p.ct_labels = s->ct_labels;
    return p;
}

// Build the kernel arguments (TMA maps for both parities, destinations).
static asets_status setup_kernel(asets_solver *s, int exact, int tile_config, bool single)
{
    const StencilVariant *v = pick_variant(s, exact, tile_config, single);
    if (!v)
        return fail(ASETS_ERR_UNSUPPORTED, "no kernel variant for this configuration");
    if (s->variant == v)
        return ASETS_OK;
    if (v->persistent && persistent_slots(s, v) < 1)
        return fail(ASETS_ERR_UNSUPPORTED, "whole-solve kernel does not fit on an SM");
    const StencilProblem p = stencil_problem_of(s, v->epi == EPI_FUSED);
    ProblemDesc &A = s->desc;
    int r = build_problem_desc(s->ctx->encode, *v, p, &A);
    if (r)
        return fail(ASETS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", r);

    const int smem = launch_smem(s, v);
    CU_TRY(cudaFuncSetAttribute(v->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, attr_smem(v)));
    int per_sm = 0;
    CU_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v->fn, v->nt, smem));
    if (per_sm < 1)
        return fail(ASETS_ERR_UNSUPPORTED, "stencil kernel does not fit on an SM");
    const long long slots = (long long)s->ctx->num_sms * per_sm;
    A.zchunks = choose_zchunks(p, *v, slots);
    const int items = problem_items(p, *v, A.zchunks);
    A.item_begin = 0;
    A.n_items = items;
    s->grid = (int)std::max<long long>(1, std::min<long long>(items, slots));
    if (!s->d_desc) {
        void *ptr = nullptr;
        CU_TRY(cudaMalloc(&ptr, sizeof(ProblemDesc)));
        s->allocations.push_back(ptr);
        s->d_desc = static_cast<ProblemDesc *>(ptr);
        CU_TRY(cudaMalloc(&ptr, 4 * sizeof(unsigned int)));
        s->allocations.push_back(ptr);
        s->d_queue = static_cast<unsigned int *>(ptr);
    }
    if (items > s->items_cap) {
        void *ptr = nullptr;
        CU_TRY(cudaMalloc(&ptr, sizeof(int) * items));
        s->allocations.push_back(ptr);
        s->d_item_problem = static_cast<int *>(ptr);
        CU_TRY(cudaMemsetAsync(s->d_item_problem, 0, sizeof(int) * items, s->ctx->stream));
        // two erriter partials per item (a two-iteration pass)
        CU_TRY(cudaMalloc(&ptr, sizeof(double) * 2 * items));
        s->allocations.push_back(ptr);
        s->d_item_partials = static_cast<double *>(ptr);
        s->items_cap = items;
    }
    A.ctl = s->ctl;
    A.item_partials = s->d_item_partials;
    s->bargs.probs = s->d_desc;
    s->bargs.item_problem = s->d_item_problem;
    s->bargs.total_items = items;
    s->bargs.queue = s->d_queue;
    s->bargs.done_count = s->d_queue + 2;
    if (v->persistent)
        s->grid = (int)std::min<long long>(items, slots);  // all resident, one or more tiles each
    // erriter partials of the label kernels (labelled models)
    const int need = std::max(s->ctx->num_sms * 8, 1024);
    if (need > s->partials_cap) {
        void *ptr = nullptr;
        CU_TRY(cudaMalloc(&ptr, sizeof(double) * need));
        s->allocations.push_back(ptr);
        s->partials = static_cast<double *>(ptr);
        s->partials_cap = need;
    }
    s->variant = v;
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_solver_create(asets_context *ctx, asets_model model,
                                                      int dim, int Ny, int Nx, int Nz, int nLab,
                                                      asets_solver **out)
{
    if (!ctx || !out)
        return fail(ASETS_ERR_INVALID_ARG, "ctx/out is NULL");
    *out = nullptr;
    if (dim != 2 && dim != 3)
        return fail(ASETS_ERR_INVALID_ARG, "dim must be 2 or 3");
    if (Ny < 1 || Nx < 1 || Nz < 1 || (dim == 2 && Nz != 1))
        return fail(ASETS_ERR_INVALID_ARG, "bad grid size %d x %d x %d", Ny, Nx, Nz);
    if (model == ASETS_BINARY) {
        nLab = 1;
    } else if (model == ASETS_POTTS) {
        if (nLab < 1)
            return fail(ASETS_ERR_INVALID_ARG, "Potts needs nLab >= 1");
    } else if (model == ASETS_ISHIKAWA) {
        if (nLab < 2)
            return fail(ASETS_ERR_INVALID_ARG, "Ishikawa needs nLab >= 2");
    } else {
        return fail(ASETS_ERR_INVALID_ARG, "unknown model %d", (int)model);
    }
    if ((long long)Ny * Nx * Nz * nLab > (1LL << 31) - 1)
        return fail(ASETS_ERR_INVALID_ARG, "problem too large for 32-bit Matlab indexing");
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    DeviceGuard guard(ctx->device);
    std::unique_ptr<asets_solver> s(new asets_solver);
    s->ctx = ctx;
    s->model = model;
    s->dim = dim;
    s->ny = Ny;
    s->nx = Nx;
    s->nz = Nz;
    s->nlab = nLab;
    s->nr = Ny;
    s->nc = (dim == 3) ? Nx : 1;
    s->ns = (dim == 3) ? Nz : Nx;
    s->pitch = round_pitch(Ny);
    s->plane = s->pitch * s->nc;
    s->cells = s->plane * s->ns;
    if (s->cells * std::max(nLab, 1) >= (1LL << 32))
        return fail(ASETS_ERR_INVALID_ARG, "padded problem exceeds 2^32 voxel-labels");
    switch (model) {
    case ASETS_BINARY:
        s->flow_labels = s->alpha_labels = s->ct_labels = s->pt_labels = s->u_labels = 1;
        break;
    case ASETS_POTTS:
        s->flow_labels = s->alpha_labels = s->ct_labels = s->pt_labels = s->u_labels = nLab;
        break;
    case ASETS_ISHIKAWA:
        s->flow_labels = s->alpha_labels = s->u_labels = nLab - 1;
        s->ct_labels = s->pt_labels = nLab;
        break;
    }
    const size_t n = (size_t)s->cells;
    asets_status st = ASETS_OK;
#define ALLOC(ptr, cnt)                      \
    do {                                     \
        st = dalloc(s.get(), &(ptr), (cnt)); \
        if (st != ASETS_OK)                  \
            goto cleanup;                    \
    } while (0)
    if (model == ASETS_BINARY)
        ALLOC(s->cs, n);
    ALLOC(s->ct, n * s->ct_labels);
    ALLOC(s->alpha, n * s->alpha_labels);
    for (int par = 0; par < 2; ++par)
        for (int k = 0; k < 3; ++k) {
            if (dim == 2 && k == 0)
                continue;
            ALLOC(s->b[par][k], n * s->flow_labels);
        }
    if (dim == 2) {
        // column faces do not exist in 2D; keep a valid pointer for the maps
        s->b[0][0] = s->b[0][1];
        s->b[1][0] = s->b[1][1];
    }
    if (model == ASETS_BINARY) {
        for (int par = 0; par < 2; ++par) {
            ALLOC(s->ps[par], n);
            ALLOC(s->pt[par], n);
            ALLOC(s->u[par], n);
        }
    } else {
        if (model == ASETS_POTTS)
            ALLOC(s->ps[0], n);
        ALLOC(s->pt[0], n * s->pt_labels);
        ALLOC(s->u[0], n * s->u_labels);
        ALLOC(s->dv, n * s->flow_labels);
        if (dim == 2 && fused2d_variant((int)model, nLab, 0)) {
            // the one-pass kernel writes the new state to a second parity
            if (model == ASETS_POTTS)
                ALLOC(s->ps[1], n);
            ALLOC(s->pt[1], n * s->pt_labels);
            ALLOC(s->u[1], n * s->u_labels);
        } else {
            s->ps[1] = s->ps[0];
            s->pt[1] = s->pt[0];
            s->u[1] = s->u[0];
        }
    }
    {
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, sizeof(IterControl));
        if (e != cudaSuccess) {
            st = cuda_fail(e, "cudaMalloc");
            goto cleanup;
        }
        s->allocations.push_back(p);
        s->ctl = static_cast<IterControl *>(p);
    }
    if (cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->flag_ev[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->flag_ev[1], cudaEventDisableTiming) != cudaSuccess) {
        st = fail(ASETS_ERR_CUDA, "cudaEventCreate failed");
        goto cleanup;
    }
#undef ALLOC
    *out = s.release();
    return ASETS_OK;
cleanup:
    asets_solver_destroy(s.release());
    return st;
}

// Copy a Matlab-layout array (rows of nr floats) into / out of the padded
// layout (rows of pitch floats).
static cudaError_t copy_in(asets_solver *s, float *dst, const float *src, int labels,
                           asets_memory where)
{
    const size_t rows = (size_t)s->nc * s->ns * labels;
    return cudaMemcpy2DAsync(dst, s->pitch * sizeof(float), src, s->nr * sizeof(float),
                             s->nr * sizeof(float), rows,
                             where == ASETS_DEVICE ? cudaMemcpyDeviceToDevice
                                                   : cudaMemcpyHostToDevice,
                             s->ctx->stream);
}

static cudaError_t copy_out(asets_solver *s, float *dst, const float *src, int labels,
                            asets_memory where)
{
    const size_t rows = (size_t)s->nc * s->ns * labels;
    return cudaMemcpy2DAsync(dst, s->nr * sizeof(float), src, s->pitch * sizeof(float),
                             s->nr * sizeof(float), rows,
                             where == ASETS_DEVICE ? cudaMemcpyDeviceToDevice
                                                   : cudaMemcpyDeviceToHost,
                             s->ctx->stream);
}

static InitArgs init_args(asets_solver *s)
{
    InitArgs a;
    memset(&a, 0, sizeof a);
    a.cs = s->cs;
    a.ct = s->ct;
    a.alpha = s->alpha;
    a.u = s->u[0];
    a.ps = s->ps[0];
    a.pt = s->pt[0];
    a.ctl = s->ctl;
    a.cells = s->cells;
    a.label_stride = s->cells;
    a.pitch = (int)s->pitch;
    a.nr = s->nr;
    a.nlab = s->nlab;
    a.alpha_labels = s->alpha_labels;
    return a;
}

extern "C" ASETS_API asets_status asets_solver_set_inputs(asets_solver *s, asets_memory where,
                                                          const float *Cs, const float *Ct,
                                                          const float *alpha)
{
    if (!s)
        return fail(ASETS_ERR_INVALID_ARG, "solver is NULL");
    if (!Ct || !alpha || (s->model == ASETS_BINARY && !Cs))
        return fail(ASETS_ERR_INVALID_ARG, "missing input array");
    std::lock_guard<std::recursive_mutex> lock(s->ctx->mu);
    DeviceGuard guard(s->ctx->device);
    if (s->model == ASETS_BINARY)
        CU_TRY(copy_in(s, s->cs, Cs, 1, where));
    CU_TRY(copy_in(s, s->ct, Ct, s->ct_labels, where));
    CU_TRY(copy_in(s, s->alpha, alpha, s->alpha_labels, where));
    // alpha(x) > 0 is checked once per input set; run() reports it when it
    // iterates, as projStep does on the first iteration.
    IterControl zero;
    memset(&zero, 0, sizeof zero);
    CU_TRY(cudaMemcpyAsync(s->ctl, &zero, sizeof zero, cudaMemcpyHostToDevice, s->ctx->stream));
    InitArgs a = init_args(s);
    CU_TRY(launch_validate_alpha(a, s->ctx->num_sms, s->ctx->stream));
    int bad = 0;
    CU_TRY(cudaMemcpyAsync(&bad, &s->ctl->alpha_bad, sizeof(int), cudaMemcpyDeviceToHost,
                           s->ctx->stream));
    CU_TRY(cudaStreamSynchronize(s->ctx->stream));
    s->alpha_ok = (bad == 0);
    s->inputs_set = true;
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_solver_get_inputs(asets_solver *s, asets_memory where,
                                                          float *Cs, float *Ct, float *alpha)
{
    if (!s)
        return fail(ASETS_ERR_INVALID_ARG, "solver is NULL");
    if (!s->inputs_set)
        return fail(ASETS_ERR_INVALID_ARG, "inputs not set");
    if (Cs && s->model != ASETS_BINARY)
        return fail(ASETS_ERR_INVALID_ARG, "only the binary model has Cs");
    std::lock_guard<std::recursive_mutex> lock(s->ctx->mu);
    DeviceGuard guard(s->ctx->device);
    if (Cs)
        CU_TRY(copy_out(s, Cs, s->cs, 1, where));
    if (Ct)
        CU_TRY(copy_out(s, Ct, s->ct, s->ct_labels, where));
    if (alpha)
        CU_TRY(copy_out(s, alpha, s->alpha, s->alpha_labels, where));
    CU_TRY(cudaStreamSynchronize(s->ctx->stream));
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_solver_set_initial(asets_solver *s, asets_memory where,
                                                           const float *u0, const float *ps0,
                                                           const float *pt0)
{
    if (!s)
        return fail(ASETS_ERR_INVALID_ARG, "solver is NULL");
    std::lock_guard<std::recursive_mutex> lock(s->ctx->mu);
    DeviceGuard guard(s->ctx->device);
    if (!u0 && !ps0 && !pt0) {
        s->warm = false;
        s->warm_flows = false;
        return ASETS_OK;
    }
    const bool need_ps = (s->model != ASETS_ISHIKAWA);
    if (!u0 || !pt0 || (need_ps && !ps0))
        return fail(ASETS_ERR_INVALID_ARG, "warm start needs u0, pt0%s", need_ps ? " and ps0" : "");
    const size_t n = (size_t)s->cells;
    asets_status st;
    if (!s->warm_u) {
        if ((st = dalloc(s, &s->warm_u, n * s->u_labels)) != ASETS_OK)
            return st;
        if ((st = dalloc(s, &s->warm_pt, n * s->pt_labels)) != ASETS_OK)
            return st;
        if (need_ps && (st = dalloc(s, &s->warm_ps, n)) != ASETS_OK)
            return st;
    }
    CU_TRY(copy_in(s, s->warm_u, u0, s->u_labels, where));
    CU_TRY(copy_in(s, s->warm_pt, pt0, s->pt_labels, where));
    if (need_ps)
        CU_TRY(copy_in(s, s->warm_ps, ps0, 1, where));
    s->warm = true;
    return ASETS_OK;
}

// Reference flow array (bx, by, bz) -> flow slot of the kernel view.  In 2D
// the stream axis is Matlab x, so bx lives in the stream-face slot.
static int flow_slot(const asets_solver *s, int ref_axis)
{
    if (ref_axis == 1)
        return SL_BR;
    if (ref_axis == 0)
        return s->dim == 3 ? SL_BC : SL_BS;
    return SL_BS;  // bz, 3D only
}

// Zero the border faces of a padded flow array (the faces at index 0 of its
// axis lie outside the volume and are never updated).
static cudaError_t zero_border_faces(asets_solver *s, float *b, int slot)
{
    const size_t L = (size_t)s->flow_labels;
    cudaStream_t st = s->ctx->stream;
    if (slot == SL_BR)
        return cudaMemset2DAsync(b, s->pitch * sizeof(float), 0, sizeof(float),
                                 (size_t)s->nc * s->ns * L, st);
    if (slot == SL_BC)
        return cudaMemset2DAsync(b, s->plane * sizeof(float), 0, s->nr * sizeof(float),
                                 (size_t)s->ns * L, st);
    return cudaMemset2DAsync(b, s->cells * sizeof(float), 0, s->plane * sizeof(float), L, st);
}

extern "C" ASETS_API asets_status asets_solver_set_initial_flows(asets_solver *s,
                                                                 asets_memory where,
                                                                 const float *bx,
                                                                 const float *by,
                                                                 const float *bz)
{
    if (!s)
        return fail(ASETS_ERR_INVALID_ARG, "solver is NULL");
    std::lock_guard<std::recursive_mutex> lock(s->ctx->mu);
    DeviceGuard guard(s->ctx->device);
    if (!bx && !by && !bz) {
        s->warm_flows = false;
        return ASETS_OK;
    }
    if (!bx || !by || (s->dim == 3) != (bz != nullptr))
        return fail(ASETS_ERR_INVALID_ARG, "initial flows need bx, by%s", s->dim == 3 ? " and bz" : " (and no bz)");
    const size_t n = (size_t)s->cells * s->flow_labels;
    const float *src[3] = {bx, by, bz};
    for (int a = 0; a < s->dim; ++a) {
        const int k = flow_slot(s, a);
        if (!s->warm_b[k]) {
            asets_status st = dalloc(s, &s->warm_b[k], n);
            if (st != ASETS_OK)
                return st;
        }
        CU_TRY(copy_in(s, s->warm_b[k], src[a], s->flow_labels, where));
        CU_TRY(zero_border_faces(s, s->warm_b[k], k));
    }
    s->warm_flows = true;
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_solver_get_spatial_flows(asets_solver *s,
                                                                 asets_memory where, float *bx,
                                                                 float *by, float *bz)
{
    if (!s)
        return fail(ASETS_ERR_INVALID_ARG, "NULL solver");
    if (bz && s->dim == 2)
        return fail(ASETS_ERR_INVALID_ARG, "a 2D problem has no bz");
    std::lock_guard<std::recursive_mutex> lock(s->ctx->mu);
    DeviceGuard guard(s->ctx->device);
    float *dst[3] = {bx, by, bz};
    for (int a = 0; a < s->dim; ++a)
        if (dst[a])
            CU_TRY(copy_out(s, dst[a], s->b[s->flow_parity][flow_slot(s, a)], s->flow_labels, where));
    CU_TRY(cudaStreamSynchronize(s->ctx->stream));
    return ASETS_OK;
}

static cudaError_t launch_stencil(asets_solver *s)
{
    const StencilVariant *v = s->variant;
    void *params[] = {&s->bargs};
    return cudaLaunchKernel(v->fn, dim3(s->grid), dim3(v->nt), params, launch_smem(s, v),
                            s->ctx->stream);
}

static LabelArgs label_args(asets_solver *s)
{
    LabelArgs a;
    memset(&a, 0, sizeof a);
    a.u = s->u[0];
    a.pt = s->pt[0];
    a.ps = s->ps[0];
    a.dv = s->dv;
    a.ct = s->ct;
    a.ctl = s->ctl;
    a.partials = s->partials;
    a.cvg = s->cvg;
    a.cells = s->cells;
    a.label_stride = s->cells;
    a.pitch = (int)s->pitch;
    a.nr = s->nr;
    a.nlab = s->nlab;
    a.cc = s->desc.cc;
    a.inv_cc = s->desc.inv_cc;
    // `1/(cc*nLab)` of updatePSU: cc*nLab rounded to float, then divided
    a.inv_cc_l = 1.0f / (s->desc.cc * (float)s->nlab);
    a.rows = (unsigned int)(s->cells / s->pitch);
    a.exact = s->variant ? s->variant->exact : 1;
    return a;
}

// Reset the solver's iteration state for a run of maxIt iterations and queue
// its initial state (zero flows; u/ps/pt from init or the warm start).
static asets_status prepare_run(asets_solver *s, int flags, int tile_config, int maxIt,
                                float errBound, float cc, float steps, bool single = true)
{
    cudaStream_t st = s->ctx->stream;
    if (maxIt >= 1 && !s->alpha_ok && !(flags & ASETS_FLAG_NO_ALPHA_CHECK))
        return fail(ASETS_ERR_ALPHA, "%s", s->alpha_labels > 1 && s->model != ASETS_BINARY
                                               ? "alpha(x,l) must be positive. Exiting..."
                                               : "alpha(x) must be positive. Exiting...");
    const int exact = (flags & ASETS_FLAG_EXACT) ? 1 : 0;
    asets_status ss = setup_kernel(s, exact, tile_config, single);
    if (ss != ASETS_OK)
        return ss;
    if (maxIt + 1 > s->cvg_cap) {
        // one spare slot past maxIt: the erriter of a roll-back re-run
        float *p = nullptr;
        ss = dalloc(s, &p, (size_t)maxIt + 1);
        if (ss != ASETS_OK)
            return ss;
        s->cvg = p;
        s->cvg_cap = maxIt + 1;
    }
    ProblemDesc &A = s->desc;
    A.cvg = s->cvg;
    A.cc = cc;
    A.inv_cc = 1.0f / cc;  // `1/cc` of the reference, a float division
    // `1/(cc*nLab)` of updatePSU: cc*nLab rounded to float, then divided
    A.inv_cc_l = 1.0f / (cc * (float)s->nlab);
    A.steps = steps;
    CU_TRY(cudaMemcpyAsync(s->d_desc, &A, sizeof A, cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemsetAsync(s->d_queue, 0, 4 * sizeof(unsigned int), st));

    IterControl c;
    memset(&c, 0, sizeof c);
    c.done = (maxIt == 0) ? 1 : 0;
    c.last_iter = -1;
    c.max_it = maxIt;
    c.err_bound = errBound;
    c.break_lt = (s->model == ASETS_ISHIKAWA && s->dim == 2) ? 1 : 0;
    c.denom = (float)(int)((long long)s->ny * s->nx * s->nz * s->u_labels);  // (float)(Nx*Ny*Nz[*L])
    CU_TRY(cudaMemcpyAsync(s->ctl, &c, sizeof c, cudaMemcpyHostToDevice, st));
    if (maxIt > 0)
        CU_TRY(cudaMemsetAsync(s->cvg, 0, sizeof(float) * maxIt, st));

    const size_t n = (size_t)s->cells;
    for (int k = 0; k < 3; ++k) {
        if (s->dim == 2 && k == 0)
            continue;
        if (s->warm_flows)
            CU_TRY(cudaMemcpyAsync(s->b[0][k], s->warm_b[k], n * s->flow_labels * sizeof(float),
                                   cudaMemcpyDeviceToDevice, st));
        else
            CU_TRY(cudaMemsetAsync(s->b[0][k], 0, n * s->flow_labels * sizeof(float), st));
    }
    if (s->warm) {
        CU_TRY(cudaMemcpyAsync(s->u[0], s->warm_u, n * s->u_labels * sizeof(float),
                               cudaMemcpyDeviceToDevice, st));
        CU_TRY(cudaMemcpyAsync(s->pt[0], s->warm_pt, n * s->pt_labels * sizeof(float),
                               cudaMemcpyDeviceToDevice, st));
        if (s->warm_ps)
            CU_TRY(cudaMemcpyAsync(s->ps[0], s->warm_ps, n * sizeof(float),
                                   cudaMemcpyDeviceToDevice, st));
    } else {
        InitArgs ia = init_args(s);
        CU_TRY(launch_init((int)s->model, ia, s->ctx->num_sms, st));
    }
    s->last_max_it = maxIt;
    return ASETS_OK;
}

// Kernels of one ALM iteration of a single solver.
static cudaError_t launch_iteration(asets_solver *s)
{
    cudaError_t e = launch_stencil(s);
    if (e != cudaSuccess || s->model == ASETS_BINARY || s->variant->epi == EPI_FUSED)
        return e;
    LabelArgs la = label_args(s);
    const int grid = label_kernel_grid(s->cells, s->ctx->num_sms);
    return s->model == ASETS_POTTS ? launch_potts_labels(la, grid, s->ctx->stream)
                                   : launch_ishikawa_labels(la, grid, s->ctx->stream);
}

// Iteration chunks of kGraphIters iterations are captured once into a CUDA
// graph and replayed; the kernels skip work once their problem is done.
static constexpr int kGraphIters = 16;

// The whole solve as one cooperative launch (square-tile kernels): every
// block resident, a grid barrier between iterations (the kernel stops at
// errBound or maxIt by itself).
static cudaError_t launch_persistent(asets_solver *s)
{
    const StencilVariant *v = s->variant;
    void *params[] = {&s->bargs};
    return cudaLaunchCooperativeKernel(v->fn, dim3(s->grid), dim3(v->nt), params, launch_smem(s, v),
                                       s->ctx->stream);
}


template <class LaunchOne>
static asets_status capture_chunk(ChunkGraph &g, cudaStream_t st, LaunchOne launch_one)
{
    g.reset();
    cudaGraph_t graph = nullptr;
    CU_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < kGraphIters && e == cudaSuccess; ++i)
        e = launch_one();
    cudaError_t e2 = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (graph)
            cudaGraphDestroy(graph);
        return cuda_fail(e != cudaSuccess ? e : e2, "capturing an iteration chunk");
    }
    e = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGraphInstantiate");
    return ASETS_OK;
}

// Replay chunks until `launched` reaches maxIt or the done flag read back at
// `done_dev` equals `done_target`.  At most two chunks are queued: before
// queueing chunk c the host looks at the flag copied after chunk c-2.
static asets_status run_chunks(asets_context *ctx, cudaGraphExec_t exec, int maxIt,
                               const unsigned int *done_dev, unsigned int done_target,
                               cudaEvent_t flag_ev[2], int *chunks_out, int iters_per_launch = 1)
{
    cudaStream_t st = ctx->stream;
    int *flags_h = ctx->pinned_flags;
    int launched = 0, chunk = 0;
    while (launched < maxIt) {
        if (chunk >= 2) {
            CU_TRY(cudaEventSynchronize(flag_ev[chunk % 2]));
            if ((unsigned int)flags_h[chunk % 2] >= done_target)
                break;
        }
        {
            NvtxRange r("asets iteration chunk");
            CU_TRY(cudaGraphLaunch(exec, st));
        }
        launched += kGraphIters * iters_per_launch;
        CU_TRY(cudaMemcpyAsync(&flags_h[chunk % 2], done_dev, sizeof(int), cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaEventRecord(flag_ev[chunk % 2], st));
        ++chunk;
    }
    *chunks_out = chunk;
    return ASETS_OK;
}

// Read back the control block after the run and record the result.
static asets_status finish_run(asets_solver *s, const IterControl &out, int *itNum)
{
    const int maxIt = s->last_max_it;
    if (out.error & DEV_ERR_TIMEOUT)
        return fail(ASETS_ERR_TIMEOUT, "a device-side wait for a TMA load timed out");
    if (out.error & DEV_ERR_BOUNDS)
        return fail(ASETS_ERR_CUDA, "an out-of-range store or shared-memory index was caught "
                    "(bounds-check build)");
    if (maxIt > 0 && !out.done)
        return fail(ASETS_ERR_CUDA, "iteration loop ended without completion (iter=%d)", out.iter);
    // The state after iteration k is in parity (k & 1).  With two
    // iterations per pass a pass starting at iteration it (even) reads
    // parity (it/2) & 1 and leaves its result -- or, after a roll-back, the
    // re-run first iteration's -- in the other one.
    const int parity = (s->variant && s->variant->temporal == 2)
                           ? (((out.last_iter >> 1) & 1) ^ 1)
                           : ((out.last_iter + 1) & 1);
    // the two-pass multi-label form keeps pt/u/ps in place (parity 0)
    const bool pingpong = (s->model == ASETS_BINARY) || (s->variant && s->variant->epi == EPI_FUSED);
    s->final_parity = pingpong ? parity : 0;
    s->flow_parity = parity;
    if (itNum)
        *itNum = (maxIt == 0) ? 0 : out.it_num;
    return ASETS_OK;
}

static asets_status ensure_items(asets_solver *s, int items);

// A two-iteration pass whose first iteration ended the solve (erriter met
// errBound there, or maxIt was reached) has stored the second iteration's
// state; the result is the first's.  Re-run that iteration with the
// one-iteration kernel from the state before the pass, still in the pass's
// source parity: when that parity is 1 the descriptor's parity halves are
// swapped, so that the kernel (which reads parity it & 1 = 0 for an even
// iteration) reads it and writes the other.  The re-run's erriter goes to a
// spare cvg slot and its control block is put back to the pass's decision,
// so cvg, itNum and the stopping iteration are those of the pass.
static asets_status replay_first_of_pass(asets_solver *s, const IterControl &out)
{
    const int it = out.last_iter;
    const int p = (it >> 1) & 1;
    int n = 0;
    const StencilVariant *tab = stencil_variants(s->dim, EPI_BINARY, s->variant->exact, &n);
    const StencilVariant *v = nullptr;
    for (int i = 0; i < n && !v; ++i)
        if (tab[i].temporal == 1)
            v = &tab[i];
    if (!v)
        return fail(ASETS_ERR_UNSUPPORTED, "no one-iteration kernel variant to re-run with");
    const StencilProblem sp = stencil_problem_of(s, false);
    ProblemDesc D;
    int r = build_problem_desc(s->ctx->encode, *v, sp, &D);
    if (r)
        return fail(ASETS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", r);
    CU_TRY(cudaFuncSetAttribute(v->fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                v->smem_bytes));
    int per_sm = 0;
    CU_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v->fn, v->nt, v->smem_bytes));
    if (per_sm < 1)
        return fail(ASETS_ERR_UNSUPPORTED, "stencil kernel does not fit on an SM");
    const long long slots = (long long)s->ctx->num_sms * per_sm;
    D.zchunks = choose_zchunks(sp, *v, slots);
    const int items = problem_items(sp, *v, D.zchunks);
    asets_status st = ensure_items(s, items);
    if (st != ASETS_OK)
        return st;
    D.item_begin = 0;
    D.n_items = items;
    D.ctl = s->ctl;
    D.item_partials = s->d_item_partials;
    D.cvg = s->cvg + (s->last_max_it - it);  // cvg[it] of the re-run: the spare slot cvg[maxIt]
    D.cc = s->desc.cc;
    D.inv_cc = s->desc.inv_cc;
    D.steps = s->desc.steps;
    if (p == 1) {
        std::swap(D.halo[0], D.halo[1]);
        std::swap(D.tile[0], D.tile[1]);
        std::swap(D.dst_b[0], D.dst_b[1]);
        std::swap(D.dst_s[0], D.dst_s[1]);
    }
    cudaStream_t stm = s->ctx->stream;
    if (!s->d_desc_replay) {
        void *ptr = nullptr;
        CU_TRY(cudaMalloc(&ptr, sizeof(ProblemDesc)));
        s->allocations.push_back(ptr);
        s->d_desc_replay = static_cast<ProblemDesc *>(ptr);
    }
    CU_TRY(cudaMemcpyAsync(s->d_desc_replay, &D, sizeof D, cudaMemcpyHostToDevice, stm));
    IterControl c = out;
    c.iter = it;
    c.done = 0;
    c.max_it = it + 1;
    c.err_bound = -1.0f;  // never met: the re-run ends by maxIt
    c.ticket = 0;
    c.error = 0;
    c.rollback = 0;
    CU_TRY(cudaMemcpyAsync(s->ctl, &c, sizeof c, cudaMemcpyHostToDevice, stm));
    BatchArgs ba;
    ba.probs = s->d_desc_replay;
    ba.item_problem = s->d_item_problem;
    ba.total_items = items;
    ba.queue = s->d_queue;
    ba.done_count = s->d_queue + 2;
    void *params[] = {&ba};
    const long long grid = std::max<long long>(1, std::min<long long>(items, slots));
    CU_TRY(cudaLaunchKernel(v->fn, dim3((unsigned)grid), dim3(v->nt), params, v->smem_bytes, stm));
    IterControl chk;
    CU_TRY(cudaMemcpyAsync(&chk, s->ctl, sizeof chk, cudaMemcpyDeviceToHost, stm));
    CU_TRY(cudaStreamSynchronize(stm));
    if (chk.error & DEV_ERR_TIMEOUT)
        return fail(ASETS_ERR_TIMEOUT, "a device-side wait for a TMA load timed out");
    if (!chk.done || chk.last_iter != it)
        return fail(ASETS_ERR_CUDA, "re-run of iteration %d did not complete", it);
    IterControl back = out;  // the pass's decision stands
    CU_TRY(cudaMemcpyAsync(s->ctl, &back, sizeof back, cudaMemcpyHostToDevice, stm));
    CU_TRY(cudaStreamSynchronize(stm));
    return ASETS_OK;
}

// ASETS_FLAG_AUTOTUNE for one solver: time every kernel variant of its kind
// on one chunk of iterations of this problem (each from the same initial
// state) and keep the fastest; the choice is cached per process by model,
// size and exactness.
static std::mutex g_solver_tune_mu;
static std::vector<std::pair<std::string, int>> g_solver_tune;

static asets_status solver_autotune(asets_solver *s, int flags, float cc, float steps,
                                    int *tile_config)
{
    NvtxRange nv("asets autotune");
    const int exact = (flags & ASETS_FLAG_EXACT) ? 1 : 0;
    char key[128];
    snprintf(key, sizeof key, "model%d/%dx%dx%d/L%d/exact%d", (int)s->model, s->ny, s->nx, s->nz,
             s->nlab, exact);
    {
        std::lock_guard<std::mutex> lk(g_solver_tune_mu);
        for (auto &kv : g_solver_tune)
            if (kv.first == key) {
                *tile_config = kv.second;
                return ASETS_OK;
            }
    }
    cudaStream_t st = s->ctx->stream;
    const std::vector<const StencilVariant *> cands = solver_candidates(s, exact, true);
    const int n = (int)cands.size();
    int best = 1;
    float best_ms = 1e30f;
    for (int cand = 1; cand <= n; ++cand) {
        // one chunk of launches: kGraphIters x (iterations per launch) iterations
        const int per_launch = cands[cand - 1]->temporal;
        if (cands[cand - 1]->persistent && persistent_slots(s, cands[cand - 1]) < 1)
            continue;
        asets_status ss = prepare_run(s, flags, cand, kGraphIters * per_launch, 0.0f, cc, steps);
        if (ss != ASETS_OK)
            return ss;
        if (s->variant->persistent) {
            // kGraphIters iterations in one cooperative launch
            CU_TRY(cudaEventRecord(s->ev0, st));
            CU_TRY(launch_persistent(s));
            CU_TRY(cudaEventRecord(s->ev1, st));
        } else {
            ss = capture_chunk(s->graph, st, [&] { return launch_iteration(s); });
            if (ss != ASETS_OK)
                return ss;
            CU_TRY(cudaEventRecord(s->ev0, st));
            CU_TRY(cudaGraphLaunch(s->graph.exec, st));
            CU_TRY(cudaEventRecord(s->ev1, st));
        }
        CU_TRY(cudaEventSynchronize(s->ev1));
        float ms = 0.f;
        CU_TRY(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
        ms /= (float)per_launch;  // per kGraphIters iterations
        if (ms < best_ms) {
            best_ms = ms;
            best = cand;
        }
    }
    s->graph.reset();  // the run captures its own chunk
    std::lock_guard<std::mutex> lk(g_solver_tune_mu);
    g_solver_tune.emplace_back(key, best);
    *tile_config = best;
    return ASETS_OK;
}

// Run a prepared solve whose variant is a whole-solve cooperative kernel.
static asets_status persistent_run(asets_solver *s, int maxIt, int *itNum)
{
    cudaStream_t st = s->ctx->stream;
    CU_TRY(cudaEventRecord(s->ev0, st));
    if (maxIt > 0) {
        NvtxRange r("asets cooperative solve");
        CU_TRY(launch_persistent(s));
    }
    CU_TRY(cudaEventRecord(s->ev1, st));
    IterControl out;
    CU_TRY(cudaMemcpyAsync(&out, s->ctl, sizeof out, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    float ms = 0.f;
    CU_TRY(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    s->last_ms = ms;
    s->last_launches = maxIt > 0 ? 1 : 0;
    s->last_iters = (maxIt == 0) ? 0 : out.last_iter + 1;
    return finish_run(s, out, itNum);
}

extern "C" ASETS_API asets_status asets_solver_run(asets_solver *s, const asets_options *opt,
                                                   int maxIt, float errBound, float cc,
                                                   float steps, int *itNum)
{
    if (!s)
        return fail(ASETS_ERR_INVALID_ARG, "solver is NULL");
    if (maxIt < 0)
        return fail(ASETS_ERR_INVALID_ARG, "maxIt must be >= 0");
    if (!s->inputs_set)
        return fail(ASETS_ERR_INVALID_ARG, "inputs not set");
    const int flags = opt ? opt->flags : 0;
    std::lock_guard<std::recursive_mutex> lock(s->ctx->mu);
    NvtxRange nv("asets_solver_run");
    DeviceGuard guard(s->ctx->device);
    cudaStream_t st = s->ctx->stream;
    int tile_config = opt ? opt->tile_config : 0;
    if ((flags & ASETS_FLAG_AUTOTUNE) && tile_config == 0 && maxIt > 0) {
        asets_status ts = solver_autotune(s, flags, cc, steps, &tile_config);
        if (ts != ASETS_OK)
            return ts;
    }
    asets_status ss = prepare_run(s, flags, tile_config, maxIt, errBound, cc, steps);
    if (ss != ASETS_OK)
        return ss;
    if (s->variant->persistent)
        return persistent_run(s, maxIt, itNum);
    // the labelled models pass cc by value to the label kernel: recapture
    // when it changes
    if (!s->graph.exec || s->graph.key_fn != s->variant->fn ||
        (s->model != ASETS_BINARY && (s->graph.key_cc != cc || s->graph.key_cvg != s->cvg))) {
        ss = capture_chunk(s->graph, st, [&] { return launch_iteration(s); });
        if (ss != ASETS_OK)
            return ss;
        s->graph.key_fn = s->variant->fn;
        s->graph.key_cc = cc;
        s->graph.key_cvg = s->cvg;
    }
    CU_TRY(cudaEventRecord(s->ev0, st));
    int chunks = 0;
    ss = run_chunks(s->ctx, s->graph.exec, maxIt, reinterpret_cast<const unsigned int *>(&s->ctl->done),
                    1u, s->flag_ev, &chunks, s->variant->temporal);
    if (ss != ASETS_OK)
        return ss;
    CU_TRY(cudaEventRecord(s->ev1, st));
    IterControl out;
    CU_TRY(cudaMemcpyAsync(&out, s->ctl, sizeof out, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    int replays = 0;
    if (maxIt > 0 && out.done && out.rollback && !(out.error & DEV_ERR_TIMEOUT)) {
        ss = replay_first_of_pass(s, out);
        if (ss != ASETS_OK)
            return ss;
        replays = 1;
        CU_TRY(cudaEventRecord(s->ev1, st));  // the re-run counts into the solve's time
        CU_TRY(cudaEventSynchronize(s->ev1));
    }
    float ms = 0.f;
    CU_TRY(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    s->last_ms = ms;
    const bool one_kernel = (s->model == ASETS_BINARY) || s->variant->epi == EPI_FUSED;
    s->last_launches = chunks * kGraphIters * (one_kernel ? 1 : 2) + replays;
    s->last_iters = (maxIt == 0) ? 0 : out.last_iter + 1;
    return finish_run(s, out, itNum);
}

extern "C" ASETS_API asets_status asets_solver_get_u(asets_solver *s, asets_memory where, float *u)
{
    if (!s || !u)
        return fail(ASETS_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::recursive_mutex> lock(s->ctx->mu);
    DeviceGuard guard(s->ctx->device);
    CU_TRY(copy_out(s, u, s->u[s->final_parity], s->u_labels, where));
    CU_TRY(cudaStreamSynchronize(s->ctx->stream));
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_solver_get_cvg(asets_solver *s, asets_memory where,
                                                       float *cvg, int n)
{
    if (!s || (!cvg && n > 0))
        return fail(ASETS_ERR_INVALID_ARG, "NULL argument");
    if (n < 0 || n > s->last_max_it)
        return fail(ASETS_ERR_INVALID_ARG, "n=%d exceeds maxIt of the last run (%d)", n,
                    s->last_max_it);
    if (n == 0)
        return ASETS_OK;
    std::lock_guard<std::recursive_mutex> lock(s->ctx->mu);
    DeviceGuard guard(s->ctx->device);
    CU_TRY(cudaMemcpyAsync(cvg, s->cvg, sizeof(float) * n,
                           where == ASETS_DEVICE ? cudaMemcpyDeviceToDevice
                                                 : cudaMemcpyDeviceToHost,
                           s->ctx->stream));
    CU_TRY(cudaStreamSynchronize(s->ctx->stream));
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_solver_get_flows(asets_solver *s, asets_memory where,
                                                         float *ps, float *pt)
{
    if (!s)
        return fail(ASETS_ERR_INVALID_ARG, "NULL solver");
    std::lock_guard<std::recursive_mutex> lock(s->ctx->mu);
    DeviceGuard guard(s->ctx->device);
    if (ps) {
        if (s->model == ASETS_ISHIKAWA)
            return fail(ASETS_ERR_INVALID_ARG, "the Ishikawa model has no source flow");
        CU_TRY(copy_out(s, ps, s->ps[s->final_parity], 1, where));
    }
    if (pt)
        CU_TRY(copy_out(s, pt, s->pt[s->final_parity], s->pt_labels, where));
    CU_TRY(cudaStreamSynchronize(s->ctx->stream));
    return ASETS_OK;
}

// ---------------------------------------------------------------- multilevel

static GridGeom geom_of(const asets_solver *s)
{
    GridGeom g;
    g.nr = s->nr;
    g.nc = s->nc;
    g.ns = s->ns;
    g.pitch = s->pitch;
    g.plane = s->plane;
    g.cells = s->cells;
    return g;
}

// Extend the chain of coarse solvers to `levels` levels where the grid
// allows (every coarse axis keeps at least kMinCoarseCells cells) and
// restrict the inputs down the chain.  Returns the number of levels.
static asets_status ml_prepare(asets_solver *s, int levels, int *built)
{
    asets_solver *cur = s;
    int n = 1;
    while (n < levels && n < kMaxLevels) {
        const int ny = (cur->ny + 1) / 2, nx = (cur->nx + 1) / 2;
        const int nz = cur->dim == 3 ? (cur->nz + 1) / 2 : 1;
        if (ny < kMinCoarseCells || nx < kMinCoarseCells || (cur->dim == 3 && nz < kMinCoarseCells))
            break;
        if (!cur->coarse) {
            asets_solver *c = nullptr;
            asets_status st = asets_solver_create(cur->ctx, cur->model, cur->dim, ny, nx, nz,
                                                  cur->nlab, &c);
            if (st != ASETS_OK)
                return st;
            cur->coarse = c;
        }
        asets_solver *c = cur->coarse;
        GridXfer X;
        X.f = geom_of(cur);
        X.c = geom_of(c);
        const int sms = cur->ctx->num_sms;
        cudaStream_t stm = cur->ctx->stream;
        if (cur->model == ASETS_BINARY)
            CU_TRY(launch_restrict(X, cur->cs, c->cs, 1, 2.f, sms, stm));
        CU_TRY(launch_restrict(X, cur->ct, c->ct, cur->ct_labels, 2.f, sms, stm));
        CU_TRY(launch_restrict(X, cur->alpha, c->alpha, cur->alpha_labels, 1.f, sms, stm));
        c->inputs_set = true;
        c->alpha_ok = cur->alpha_ok;
        cur = c;
        ++n;
    }
    *built = n;
    return ASETS_OK;
}

// Initial state of `f` from the solved state of the next coarser level `c`.
static asets_status ml_prolong(asets_solver *c, asets_solver *f)
{
    const size_t n = (size_t)f->cells;
    const bool has_ps = (f->model != ASETS_ISHIKAWA);
    asets_status st;
    if (!f->warm_u) {
        if ((st = dalloc(f, &f->warm_u, n * f->u_labels)) != ASETS_OK)
            return st;
        if ((st = dalloc(f, &f->warm_pt, n * f->pt_labels)) != ASETS_OK)
            return st;
        if (has_ps && (st = dalloc(f, &f->warm_ps, n)) != ASETS_OK)
            return st;
    }
    GridXfer X;
    X.f = geom_of(f);
    X.c = geom_of(c);
    const int sms = f->ctx->num_sms;
    cudaStream_t stm = f->ctx->stream;
    CU_TRY(launch_prolong(X, c->u[c->final_parity], f->warm_u, f->u_labels, 1.f, -1, sms, stm));
    CU_TRY(launch_prolong(X, c->pt[c->final_parity], f->warm_pt, f->pt_labels, 0.5f, -1, sms, stm));
    if (has_ps)
        CU_TRY(launch_prolong(X, c->ps[c->final_parity], f->warm_ps, 1, 0.5f, -1, sms, stm));
    for (int k = 0; k < 3; ++k) {
        if (f->dim == 2 && k == SL_BC)
            continue;
        if (!f->warm_b[k] && (st = dalloc(f, &f->warm_b[k], n * f->flow_labels)) != ASETS_OK)
            return st;
        const int axis = (k == SL_BR) ? 0 : (k == SL_BC ? 1 : 2);
        CU_TRY(launch_prolong(X, c->b[c->flow_parity][k], f->warm_b[k], f->flow_labels, 1.f, axis,
                              sms, stm));
    }
    f->warm = true;
    f->warm_flows = true;
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_solver_multilevel_prepare(asets_solver *s, int levels,
                                                                  int *levels_out)
{
    if (!s || levels < 1)
        return fail(ASETS_ERR_INVALID_ARG, "bad multilevel arguments");
    if (!s->inputs_set)
        return fail(ASETS_ERR_INVALID_ARG, "inputs not set");
    std::lock_guard<std::recursive_mutex> lock(s->ctx->mu);
    DeviceGuard guard(s->ctx->device);
    int built = 1;
    asets_status st = ml_prepare(s, levels, &built);
    if (st != ASETS_OK)
        return st;
    CU_TRY(cudaStreamSynchronize(s->ctx->stream));
    if (levels_out)
        *levels_out = built;
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_solver_level(asets_solver *s, int level, asets_solver **out)
{
    if (!s || !out || level < 0)
        return fail(ASETS_ERR_INVALID_ARG, "bad arguments");
    asets_solver *cur = s;
    for (int k = 0; k < level && cur; ++k)
        cur = cur->coarse;
    if (!cur)
        return fail(ASETS_ERR_INVALID_ARG, "level %d does not exist (call asets_solver_multilevel_prepare)", level);
    *out = cur;
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_solver_run_multilevel(asets_solver *s,
                                                              const asets_options *opt,
                                                              int levels, int maxIt,
                                                              float errBound, float cc,
                                                              float steps, int *itNum)
{
    if (!s || levels < 1 || maxIt < 0)
        return fail(ASETS_ERR_INVALID_ARG, "bad multilevel arguments");
    if (!s->inputs_set)
        return fail(ASETS_ERR_INVALID_ARG, "inputs not set");
    std::lock_guard<std::recursive_mutex> lock(s->ctx->mu);
    DeviceGuard guard(s->ctx->device);
    int built = 1;
    asets_status st = ml_prepare(s, levels, &built);
    if (st != ASETS_OK)
        return st;
    asets_solver *lv[kMaxLevels];
    lv[0] = s;
    for (int k = 1; k < built; ++k)
        lv[k] = lv[k - 1]->coarse;
    s->ml_levels = 0;
    for (int k = built - 1; k >= 0; --k) {
        NvtxRange nv("asets multilevel level");
        asets_solver *cur = lv[k];
        if (k < built - 1 && (st = ml_prolong(lv[k + 1], cur)) != ASETS_OK)
            return st;
        int it = 0;
        st = asets_solver_run(cur, opt, maxIt, errBound, cc, steps, &it);
        if (k < built - 1) {
            cur->warm = false;  // the prolonged state is consumed by this run
            cur->warm_flows = false;
        }
        if (st != ASETS_OK)
            return st;
        s->ml_iters[k] = it;
        s->ml_ms[k] = cur->last_ms;
    }
    s->ml_levels = built;
    if (itNum)
        *itNum = s->ml_iters[0];
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_solver_multilevel_stats(asets_solver *s, int cap,
                                                                int *iters, float *ms,
                                                                int *levels_out)
{
    if (!s)
        return fail(ASETS_ERR_INVALID_ARG, "NULL solver");
    for (int k = 0; k < s->ml_levels && k < cap; ++k) {
        if (iters)
            iters[k] = s->ml_iters[k];
        if (ms)
            ms[k] = s->ml_ms[k];
    }
    if (levels_out)
        *levels_out = s->ml_levels;
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_solver_last_run_stats(asets_solver *s, float *ms,
                                                              int *kernel_launches)
{
    if (!s)
        return fail(ASETS_ERR_INVALID_ARG, "NULL solver");
    if (ms)
        *ms = s->last_ms;
    if (kernel_launches)
        *kernel_launches = s->last_launches;
    return ASETS_OK;
}

// ---------------------------------------------------------------- batch
// Many independent problems solved together: per iteration one launch of
// the fused flow pass per group (binary / labelled x 2D / 3D) over all live
// problems' work items, then, for the labelled models, each problem's label
// kernel; each problem converges (and retires) on its own.
struct asets_batch {
    asets_context *ctx = nullptr;
    std::vector<asets_solver *> members;
    struct Group {
        std::vector<int> idx;  // members of this group
        std::vector<int> live; // members in the current layout (not yet retired)
        const StencilVariant *v = nullptr;
        ProblemDesc *d_desc = nullptr;
        int desc_cap = 0;
        int *d_item_problem = nullptr;
        int items_cap = 0;
        unsigned int *d_queue = nullptr;
        BatchArgs bargs;
        int grid = 0;
        int tile_config = 0;
    } groups[4];  // [0] binary 2D, [1] binary 3D, [2] labelled 2D, [3] labelled 3D
    unsigned int *d_done = nullptr;
    IterControl **d_ctls = nullptr;  // every member's control block
    int *d_member_done = nullptr;    // gathered done flags
    int *h_member_done = nullptr;    // pinned copy
    int ctls_cap = 0;
    ChunkGraph graph;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, flag_ev[2] = {nullptr, nullptr};
    std::vector<void *> allocations;
    float last_ms = 0.f;
    int last_launches = 0;
    asets_batch *level[kMaxLevels] = {};  // multilevel runs: the members' coarse levels
};

// done counter, then three queue words per group
static constexpr int kBatchCounters = 16;

static int batch_group(const asets_solver *s)
{
    return (s->dim == 3 ? 1 : 0) + (s->model == ASETS_BINARY ? 0 : 2);
}

extern "C" ASETS_API asets_status asets_batch_create(asets_context *ctx, asets_batch **out)
{
    if (!ctx || !out)
        return fail(ASETS_ERR_INVALID_ARG, "ctx/out is NULL");
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    DeviceGuard guard(ctx->device);
    std::unique_ptr<asets_batch> b(new asets_batch);
    b->ctx = ctx;
    void *p = nullptr;
    CU_TRY(cudaMalloc(&p, kBatchCounters * sizeof(unsigned int)));
    b->allocations.push_back(p);
    b->d_done = static_cast<unsigned int *>(p);
    for (int g = 0; g < 4; ++g)
        b->groups[g].d_queue = b->d_done + 4 + 3 * g;
    CU_TRY(cudaEventCreate(&b->ev0));
    CU_TRY(cudaEventCreate(&b->ev1));
    CU_TRY(cudaEventCreateWithFlags(&b->flag_ev[0], cudaEventDisableTiming));
    CU_TRY(cudaEventCreateWithFlags(&b->flag_ev[1], cudaEventDisableTiming));
    *out = b.release();
    return ASETS_OK;
}

extern "C" ASETS_API void asets_batch_destroy(asets_batch *b)
{
    if (!b)
        return;
    for (asets_batch *lb : b->level)
        asets_batch_destroy(lb);
    DeviceGuard guard(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    b->graph.reset();
    for (void *p : b->allocations)
        cudaFree(p);
    if (b->h_member_done)
        cudaFreeHost(b->h_member_done);
    for (cudaEvent_t e : {b->ev0, b->ev1, b->flag_ev[0], b->flag_ev[1]})
        if (e)
            cudaEventDestroy(e);
    delete b;
}

extern "C" ASETS_API asets_status asets_batch_add(asets_batch *b, asets_solver *s)
{
    if (!b || !s)
        return fail(ASETS_ERR_INVALID_ARG, "NULL argument");
    if (s->ctx != b->ctx)
        return fail(ASETS_ERR_INVALID_ARG, "solver belongs to another context");
    for (asets_solver *m : b->members)
        if (m == s)
            return fail(ASETS_ERR_INVALID_ARG, "solver already in the batch");
    b->members.push_back(s);
    b->graph.reset();
    return ASETS_OK;
}

// Per-item partial storage of a member sized for `items`.  The member's
// own item map (used when it is solved alone) must stay all zeros: a later
// single solve may adopt the grown buffers.
static asets_status ensure_items(asets_solver *s, int items)
{
    if (items <= s->items_cap)
        return ASETS_OK;
    void *ptr = nullptr;
    CU_TRY(cudaMalloc(&ptr, sizeof(int) * items));
    s->allocations.push_back(ptr);
    s->d_item_problem = static_cast<int *>(ptr);
    CU_TRY(cudaMemsetAsync(s->d_item_problem, 0, sizeof(int) * items, s->ctx->stream));
    CU_TRY(cudaMalloc(&ptr, sizeof(double) * 2 * items));
    s->allocations.push_back(ptr);
    s->d_item_partials = static_cast<double *>(ptr);
    s->items_cap = items;
    return ASETS_OK;
}

static asets_status batch_buffer(asets_batch *b, void **p, size_t bytes)
{
    CU_TRY(cudaMalloc(p, bytes));
    b->allocations.push_back(*p);
    return ASETS_OK;
}

static StencilProblem item_geometry(const asets_solver *s)
{
    StencilProblem sp;
    memset(&sp, 0, sizeof sp);
    sp.nr = s->nr;
    sp.nc = s->nc;
    sp.ns = s->ns;
    sp.flow_labels = s->flow_labels;
    return sp;
}

// Stream-axis chunk counts for the problems of one launch: one common chunk
// length (planes per item) for all of them, the one with the best
// (wave fill of `slots` resident blocks) x (useful planes / swept planes,
// each chunk sweeping 4 warm-up planes).  Many live problems keep long
// chunks; a few left iterating (the tail of a batch) get short ones, so
// their items still spread over every SM.
static std::vector<int> choose_batch_chunks(const std::vector<asets_solver *> &live,
                                            const StencilVariant &v, long long slots)
{
    static const int kLengths[] = {8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256, 512, 1024, 4096};
    std::vector<int> best(live.size(), 1), cur(live.size(), 1);
    double best_eff = -1.0;
    for (int len : kLengths) {
        long long items = 0;
        double useful = 0.0, swept = 0.0;
        for (size_t j = 0; j < live.size(); ++j) {
            const asets_solver *s = live[j];
            const int max_k = std::max(1, s->ns / 8);
            const int k = v.s_tile > 0 ? (s->ns + v.s_tile - 1) / v.s_tile  // square tiles
                                       : std::min(max_k, std::max(1, (s->ns + len / 2) / len));
            cur[j] = k;
            const long long it = problem_items(item_geometry(s), v, k);
            items += it;
            useful += (double)it / k * s->ns;
            swept += (double)it / k * (s->ns + 4.0 * k);
        }
        if (items < 1)
            continue;
        const long long waves = (items + slots - 1) / slots;
        const double eff = ((double)items / (double)(waves * slots)) * (useful / swept);
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = cur;
        }
    }
    return best;
}

// Lay out one group's descriptors and item map for a run, over the members
// in g.live (all of the group's members at the start of a run; the ones
// still iterating when the batch re-lays itself out).
static asets_status batch_layout(asets_batch *b, asets_batch::Group &g)
{
    if (g.live.empty())
        return ASETS_OK;
    int per_sm = 0;
    CU_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, g.v->fn, g.v->nt,
                                                         g.v->smem_bytes));
    const long long slots = (long long)b->ctx->num_sms * std::max(per_sm, 1);
    std::vector<asets_solver *> live;
    for (int i : g.live)
        live.push_back(b->members[i]);
    const std::vector<int> zc = choose_batch_chunks(live, *g.v, slots);
    std::vector<ProblemDesc> descs;
    std::vector<int> item_problem;
    for (size_t j = 0; j < live.size(); ++j) {
        asets_solver *s = live[j];
        // The batch's layout lives only in its own descriptor copy `d`: the
        // member's descriptor keeps its single-solve layout, which a later
        // solve of the member alone uploads as it is.
        ProblemDesc d = s->desc;
        d.zchunks = zc[j];
        const int items = problem_items(item_geometry(s), *g.v, d.zchunks);
        asets_status st = ensure_items(s, items);
        if (st != ASETS_OK)
            return st;
        d.item_begin = (int)item_problem.size();
        d.n_items = items;
        d.item_partials = s->d_item_partials;
        item_problem.insert(item_problem.end(), items, (int)j);
        descs.push_back(d);
    }
    cudaStream_t st = b->ctx->stream;
    if ((int)descs.size() > g.desc_cap) {
        void *p = nullptr;
        asets_status s2 = batch_buffer(b, &p, sizeof(ProblemDesc) * descs.size());
        if (s2 != ASETS_OK)
            return s2;
        g.d_desc = static_cast<ProblemDesc *>(p);
        g.desc_cap = (int)descs.size();
    }
    if ((int)item_problem.size() > g.items_cap) {
        void *p = nullptr;
        asets_status s2 = batch_buffer(b, &p, sizeof(int) * item_problem.size());
        if (s2 != ASETS_OK)
            return s2;
        g.d_item_problem = static_cast<int *>(p);
        g.items_cap = (int)item_problem.size();
    }
    CU_TRY(cudaMemcpyAsync(g.d_desc, descs.data(), sizeof(ProblemDesc) * descs.size(),
                           cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(g.d_item_problem, item_problem.data(), sizeof(int) * item_problem.size(),
                           cudaMemcpyHostToDevice, st));
    CU_TRY(cudaStreamSynchronize(st));  // host vectors go out of scope
    g.grid = (int)std::min<long long>((long long)item_problem.size(), slots);
    g.bargs.probs = g.d_desc;
    g.bargs.item_problem = g.d_item_problem;
    g.bargs.total_items = (int)item_problem.size();
    g.bargs.queue = g.d_queue;
    g.bargs.done_count = b->d_done;
    return ASETS_OK;
}

static cudaError_t batch_launch_iteration(asets_batch *b)
{
    for (int gi = 0; gi < 4; ++gi) {
        auto &g = b->groups[gi];
        if (g.live.empty())
            continue;
        void *params[] = {&g.bargs};
        cudaError_t e = cudaLaunchKernel(g.v->fn, dim3(g.grid), dim3(g.v->nt), params,
                                         g.v->smem_bytes, b->ctx->stream);
        if (e != cudaSuccess)
            return e;
        if (gi < 2)
            continue;
        // labelled models: each problem's label kernel closes its iteration
        // (it returns at once for a finished problem) and counts it when done
        for (int i : g.live) {
            asets_solver *s = b->members[i];
            LabelArgs la = label_args(s);
            la.done_count = b->d_done;
            const int grid = label_kernel_grid(s->cells, s->ctx->num_sms);
            e = s->model == ASETS_POTTS ? launch_potts_labels(la, grid, b->ctx->stream)
                                        : launch_ishikawa_labels(la, grid, b->ctx->stream);
            if (e != cudaSuccess)
                return e;
        }
    }
    return cudaSuccess;
}

// Prepare every member and lay out the groups for the given tile configs.
static asets_status batch_prepare(asets_batch *b, int flags, const int tile_config[4], int maxIt,
                                  float errBound, float cc, float steps)
{
    for (auto &g : b->groups) {
        g.idx.clear();
        g.v = nullptr;
    }
    for (size_t i = 0; i < b->members.size(); ++i) {
        asets_solver *s = b->members[i];
        if (!s->inputs_set)
            return fail(ASETS_ERR_INVALID_ARG, "batch member %zu has no inputs", i);
        const int gi = batch_group(s);
        asets_status st =
            prepare_run(s, flags, tile_config[gi], maxIt, errBound, cc, steps, false);
        if (st != ASETS_OK)
            return st;
        b->groups[gi].idx.push_back((int)i);
        b->groups[gi].v = s->variant;
        b->groups[gi].tile_config = tile_config[gi];
    }
    cudaStream_t st = b->ctx->stream;
    CU_TRY(cudaMemsetAsync(b->d_done, 0, kBatchCounters * sizeof(unsigned int), st));
    const int nm = (int)b->members.size();
    if (nm > b->ctls_cap) {
        void *p = nullptr;
        asets_status s2 = batch_buffer(b, &p, sizeof(IterControl *) * nm);
        if (s2 != ASETS_OK)
            return s2;
        b->d_ctls = static_cast<IterControl **>(p);
        if ((s2 = batch_buffer(b, &p, sizeof(int) * nm)) != ASETS_OK)
            return s2;
        b->d_member_done = static_cast<int *>(p);
        if (b->h_member_done)
            cudaFreeHost(b->h_member_done);
        b->h_member_done = nullptr;
        CU_TRY(cudaMallocHost(&b->h_member_done, sizeof(int) * nm));
        b->ctls_cap = nm;
    }
    {
        std::vector<IterControl *> ctls(nm);
        for (int i = 0; i < nm; ++i)
            ctls[i] = b->members[i]->ctl;
        CU_TRY(cudaMemcpyAsync(b->d_ctls, ctls.data(), sizeof(IterControl *) * nm,
                               cudaMemcpyHostToDevice, st));
        CU_TRY(cudaStreamSynchronize(st));
    }
    for (auto &g : b->groups) {
        g.live = g.idx;
        asets_status s2 = batch_layout(b, g);
        if (s2 != ASETS_OK)
            return s2;
    }
    return ASETS_OK;
}

__global__ void gather_done_kernel(IterControl *const *ctls, int n, int *out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = *(const volatile int *)&ctls[i]->done;
}

// After members have retired: drop them from the layout of their group and
// re-choose the live members' chunk counts (choose_batch_chunks), so that
// the items of the problems still iterating cover the GPU again.  The
// stream is drained first (the descriptors are rewritten).  *changed tells
// whether a layout changed (the iteration chunk must be captured anew).
static asets_status batch_relayout(asets_batch *b, bool *changed)
{
    *changed = false;
    cudaStream_t st = b->ctx->stream;
    const int nm = (int)b->members.size();
    gather_done_kernel<<<1, 256, 0, st>>>(b->d_ctls, nm, b->d_member_done);
    CU_TRY(cudaGetLastError());
    CU_TRY(cudaMemcpyAsync(b->h_member_done, b->d_member_done, sizeof(int) * nm,
                           cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    for (auto &g : b->groups) {
        std::vector<int> live;
        for (int i : g.live)
            if (!b->h_member_done[i])
                live.push_back(i);
        if (live.size() == g.live.size())
            continue;
        g.live = live;
        asets_status s2 = batch_layout(b, g);
        if (s2 != ASETS_OK)
            return s2;
        *changed = true;
    }
    return ASETS_OK;
}

// Kernel launches of one iteration of the current layout: the flow pass of
// each group, plus the label kernel of each live labelled member.
static int batch_launches_per_iter(const asets_batch *b)
{
    int n = 0;
    for (int gi = 0; gi < 4; ++gi)
        if (!b->groups[gi].live.empty())
            n += 1 + (gi >= 2 ? (int)b->groups[gi].live.size() : 0);
    return n;
}

// Replay iteration chunks (as run_chunks) until every member is done or
// maxIt launches are queued.  Whenever the done count read back has grown,
// the retired members leave the layout (batch_relayout).  *chunks: chunks
// replayed; *launches (may be NULL): the kernel launches they held.
static asets_status batch_execute(asets_batch *b, int maxIt, int *chunks, int *launches)
{
    cudaStream_t st = b->ctx->stream;
    asets_status ss = capture_chunk(b->graph, st, [&] { return batch_launch_iteration(b); });
    if (ss != ASETS_OK)
        return ss;
    const unsigned int target = (unsigned int)b->members.size();
    int *flags_h = b->ctx->pinned_flags;
    unsigned int seen = 0;
    int launched = 0, chunk = 0, kernels = 0;
    while (launched < maxIt) {
        if (chunk >= 2) {
            CU_TRY(cudaEventSynchronize(b->flag_ev[chunk % 2]));
            const unsigned int done = (unsigned int)flags_h[chunk % 2];
            if (done >= target)
                break;
            if (done > seen) {
                seen = done;
                bool changed = false;
                if ((ss = batch_relayout(b, &changed)) != ASETS_OK)
                    return ss;
                if (changed) {
                    ss = capture_chunk(b->graph, st, [&] { return batch_launch_iteration(b); });
                    if (ss != ASETS_OK)
                        return ss;
                }
            }
        }
        {
            NvtxRange r("asets batch iteration chunk");
            CU_TRY(cudaGraphLaunch(b->graph.exec, st));
        }
        launched += kGraphIters;
        kernels += kGraphIters * batch_launches_per_iter(b);
        CU_TRY(cudaMemcpyAsync(&flags_h[chunk % 2], b->d_done, sizeof(int),
                               cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaEventRecord(b->flag_ev[chunk % 2], st));
        ++chunk;
    }
    *chunks = chunk;
    if (launches)
        *launches = kernels;
    return ASETS_OK;
}

// Tile configuration per dimension group, chosen by timing each candidate
// for a few iterations on this batch; cached per (group, exactness, size).
static std::mutex g_tune_mu;
static std::vector<std::pair<std::string, int>> g_tune_cache;

static asets_status batch_autotune(asets_batch *b, int flags, float cc, float steps, int tile_config[4])
{
    NvtxRange nv("asets batch autotune");
    const int exact = (flags & ASETS_FLAG_EXACT) ? 1 : 0;
    for (int gi = 0; gi < 4; ++gi) {
        long long vox = 0;
        int count = 0;
        for (asets_solver *s : b->members)
            if (batch_group(s) == gi) {
                vox += s->cells;
                ++count;
            }
        if (!count)
            continue;
        char key[96];
        snprintf(key, sizeof key, "group%d/exact%d/n%d/logvox%d", gi, exact, count,
                 (int)std::log2((double)std::max(vox, 1LL)));
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            bool found = false;
            for (auto &kv : g_tune_cache)
                if (kv.first == key) {
                    tile_config[gi] = kv.second;
                    found = true;
                }
            if (found)
                continue;
        }
        int n = 0;
        const StencilVariant *tab =
            stencil_variants((gi & 1) ? 3 : 2, gi >= 2 ? EPI_DIV : EPI_BINARY, exact, &n);
        int best = 1;
        float best_ms = 1e30f;
        for (int cand = 1; cand <= n; ++cand) {
            if (tab[cand - 1].persistent)
                continue;  // single solves only
            int tc[4] = {tile_config[0], tile_config[1], tile_config[2], tile_config[3]};
            tc[gi] = cand;
            // 2 x kGraphIters iterations of every member: two chunks of one
            // iteration per launch, or one of two (the second chunk's
            // launches then return at entry)
            asets_status st = batch_prepare(b, flags, tc, 2 * kGraphIters, 0.0f, cc, steps);
            if (st != ASETS_OK)
                return st;
            int chunks = 0;
            CU_TRY(cudaEventRecord(b->ev0, b->ctx->stream));
            st = batch_execute(b, 2 * kGraphIters, &chunks, nullptr);
            if (st != ASETS_OK)
                return st;
            CU_TRY(cudaEventRecord(b->ev1, b->ctx->stream));
            CU_TRY(cudaEventSynchronize(b->ev1));
            float ms = 0.f;
            CU_TRY(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
            if (ms < best_ms) {
                best_ms = ms;
                best = cand;
            }
        }
        tile_config[gi] = best;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache.emplace_back(key, best);
    }
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_batch_run(asets_batch *b, const asets_options *opt,
                                                  int maxIt, float errBound, float cc,
                                                  float steps, int *itNums)
{
    if (!b)
        return fail(ASETS_ERR_INVALID_ARG, "batch is NULL");
    if (maxIt < 0)
        return fail(ASETS_ERR_INVALID_ARG, "maxIt must be >= 0");
    if (b->members.empty())
        return ASETS_OK;
    const int flags = opt ? opt->flags : 0;
    std::lock_guard<std::recursive_mutex> lock(b->ctx->mu);
    DeviceGuard guard(b->ctx->device);
    NvtxRange nv("asets_batch_run");
    cudaStream_t st = b->ctx->stream;
    // one kernel variant per dimension group (default: the first)
    const int tc0 = (opt && opt->tile_config > 0) ? opt->tile_config : 1;
    int tile_config[4] = {tc0, tc0, tc0, tc0};
    if ((flags & ASETS_FLAG_AUTOTUNE) && maxIt > 0) {
        asets_status ts = batch_autotune(b, flags, cc, steps, tile_config);
        if (ts != ASETS_OK)
            return ts;
    }
    asets_status ss = batch_prepare(b, flags, tile_config, maxIt, errBound, cc, steps);
    if (ss != ASETS_OK)
        return ss;
    CU_TRY(cudaEventRecord(b->ev0, st));
    int chunks = 0, launches = 0;
    if (maxIt > 0) {
        ss = batch_execute(b, maxIt, &chunks, &launches);
        if (ss != ASETS_OK)
            return ss;
    }
    CU_TRY(cudaEventRecord(b->ev1, st));
    std::vector<IterControl> outs(b->members.size());
    for (size_t i = 0; i < b->members.size(); ++i)
        CU_TRY(cudaMemcpyAsync(&outs[i], b->members[i]->ctl, sizeof(IterControl),
                               cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    // members whose two-iteration pass ended at its first iteration
    int replays = 0;
    for (size_t i = 0; i < b->members.size(); ++i) {
        asets_solver *s = b->members[i];
        if (maxIt > 0 && outs[i].done && outs[i].rollback && !(outs[i].error & DEV_ERR_TIMEOUT)) {
            asets_status rs = replay_first_of_pass(s, outs[i]);
            if (rs != ASETS_OK)
                return rs;
            ++replays;
        }
    }
    if (replays) {
        CU_TRY(cudaEventRecord(b->ev1, st));  // the re-runs count into the batch's time
        CU_TRY(cudaEventSynchronize(b->ev1));
    }
    float ms = 0.f;
    CU_TRY(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->last_ms = ms;
    b->last_launches = launches + replays;  // flow passes, label kernels, re-runs
    b->groups[0].tile_config = tile_config[0];
    b->groups[1].tile_config = tile_config[1];
    for (size_t i = 0; i < b->members.size(); ++i) {
        asets_solver *s = b->members[i];
        s->last_ms = ms;
        s->last_iters = (maxIt == 0) ? 0 : outs[i].last_iter + 1;
        int it = 0;
        asets_status fs = finish_run(s, outs[i], &it);
        if (fs != ASETS_OK)
            return fs;
        if (itNums)
            itNums[i] = it;
    }
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_batch_last_run_stats(asets_batch *b, float *ms,
                                                             int *kernel_launches,
                                                             int *iterations, int *tile_configs)
{
    if (!b)
        return fail(ASETS_ERR_INVALID_ARG, "batch is NULL");
    if (ms)
        *ms = b->last_ms;
    if (kernel_launches)
        *kernel_launches = b->last_launches;
    if (iterations) {
        long long total = 0;
        for (asets_solver *s : b->members)
            total += s->last_iters;
        *iterations = (int)total;
    }
    if (tile_configs) {
        tile_configs[0] = b->groups[0].tile_config;
        tile_configs[1] = b->groups[1].tile_config;
    }
    return ASETS_OK;
}

// Coarse-to-fine solve of every member (asets_solver_run_multilevel for a
// batch): level k of all members that have one runs as one batch, each
// member's coarsest level from its own initial state, every finer level from
// the prolonged solution of the level below.
extern "C" ASETS_API asets_status asets_batch_run_multilevel(asets_batch *b,
                                                             const asets_options *opt,
                                                             int levels, int maxIt,
                                                             float errBound, float cc,
                                                             float steps, int *itNums)
{
    if (!b || levels < 1 || maxIt < 0)
        return fail(ASETS_ERR_INVALID_ARG, "bad multilevel arguments");
    std::lock_guard<std::recursive_mutex> lock(b->ctx->mu);
    DeviceGuard guard(b->ctx->device);
    const size_t m = b->members.size();
    std::vector<int> built(m, 1);
    std::vector<std::array<asets_solver *, kMaxLevels>> lv(m);
    int top = 0;
    for (size_t i = 0; i < m; ++i) {
        asets_solver *s = b->members[i];
        if (!s->inputs_set)
            return fail(ASETS_ERR_INVALID_ARG, "batch member %zu has no inputs", i);
        asets_status st = ml_prepare(s, levels, &built[i]);
        if (st != ASETS_OK)
            return st;
        lv[i][0] = s;
        for (int k = 1; k < built[i]; ++k)
            lv[i][k] = lv[i][k - 1]->coarse;
        s->ml_levels = 0;
        top = std::max(top, built[i]);
    }
    std::vector<int> its(m, 0);
    for (int k = top - 1; k >= 0; --k) {
        asets_batch *lb = b;
        if (k > 0) {
            if (!b->level[k]) {
                asets_status st = asets_batch_create(b->ctx, &b->level[k]);
                if (st != ASETS_OK)
                    return st;
            }
            lb = b->level[k];
            lb->members.clear();
            lb->graph.reset();
        }
        std::vector<size_t> who;
        for (size_t i = 0; i < m; ++i) {
            if (built[i] <= k)
                continue;
            if (k < built[i] - 1) {
                asets_status st = ml_prolong(lv[i][k + 1], lv[i][k]);
                if (st != ASETS_OK)
                    return st;
            }
            if (k > 0)
                lb->members.push_back(lv[i][k]);
            who.push_back(i);
        }
        std::vector<int> lit(lb->members.size(), 0);
        asets_status st = asets_batch_run(lb, opt, maxIt, errBound, cc, steps, lit.data());
        for (size_t i : who)
            if (k < built[i] - 1) {
                lv[i][k]->warm = false;  // the prolonged state is consumed by this run
                lv[i][k]->warm_flows = false;
            }
        if (st != ASETS_OK)
            return st;
        // the full-resolution batch is `b` itself: its itNums are in member order
        for (size_t j = 0; j < who.size(); ++j) {
            const size_t i = who[j];
            const int it = (k > 0) ? lit[j] : lit[i];
            b->members[i]->ml_iters[k] = it;
            b->members[i]->ml_ms[k] = lb->last_ms;
            if (k == 0)
                its[i] = it;
        }
    }
    for (size_t i = 0; i < m; ++i) {
        b->members[i]->ml_levels = built[i];
        if (itNums)
            itNums[i] = its[i];
    }
    return ASETS_OK;
}

// ---------------------------------------------------------------- one-shot
static asets_status one_shot(asets_context *ctx, const asets_options *opt, asets_model model,
                             int dim, int Ny, int Nx, int Nz, int nLab, const float *alpha,
                             const float *Cs, const float *Ct, int maxIt, float errBound, float cc,
                             float steps, float *u, float *cvg, int *itNum, float *seconds)
{
    const auto t0 = std::chrono::steady_clock::now();
    if (!ctx) {
        asets_status st = asets_default_context(&ctx);
        if (st != ASETS_OK)
            return st;
    }
    if (!alpha || !Ct || !u || (maxIt > 0 && !cvg) || (model == ASETS_BINARY && !Cs))
        return fail(ASETS_ERR_INVALID_ARG, "NULL input or output pointer");
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    asets_solver *s = ctx->cached;
    if (!s || s->model != model || s->dim != dim || s->ny != Ny || s->nx != Nx || s->nz != Nz ||
        s->nlab != (model == ASETS_BINARY ? 1 : nLab)) {
        if (s)
            asets_solver_destroy(s);
        ctx->cached = nullptr;
        asets_status st = asets_solver_create(ctx, model, dim, Ny, Nx, Nz, nLab, &s);
        if (st != ASETS_OK)
            return st;
        ctx->cached = s;
    }
    s->warm = false;
    asets_status st = asets_solver_set_inputs(s, ASETS_HOST, Cs, Ct, alpha);
    if (st != ASETS_OK)
        return st;
    int it = 0;
    st = asets_solver_run(s, opt, maxIt, errBound, cc, steps, &it);
    if (st != ASETS_OK)
        return st;
    st = asets_solver_get_u(s, ASETS_HOST, u);
    if (st != ASETS_OK)
        return st;
    st = asets_solver_get_cvg(s, ASETS_HOST, cvg, maxIt);
    if (st != ASETS_OK)
        return st;
    if (itNum)
        *itNum = it;
    if (seconds)
        *seconds = std::chrono::duration<float>(std::chrono::steady_clock::now() - t0).count();
    return ASETS_OK;
}

extern "C" ASETS_API asets_status asets_binary_mf2d(asets_context *ctx, const asets_options *opt,
                                                    const float *alpha, const float *Cs,
                                                    const float *Ct, int Nx, int Ny, int maxIt,
                                                    float errBound, float cc, float steps,
                                                    float *u, float *cvg, int *itNum,
                                                    float *seconds)
{
    return one_shot(ctx, opt, ASETS_BINARY, 2, Ny, Nx, 1, 1, alpha, Cs, Ct, maxIt, errBound, cc,
                    steps, u, cvg, itNum, seconds);
}

extern "C" ASETS_API asets_status asets_binary_mf3d(asets_context *ctx, const asets_options *opt,
                                                    const float *alpha, const float *Cs,
                                                    const float *Ct, int Nx, int Ny, int Nz,
                                                    int maxIt, float errBound, float cc,
                                                    float steps, float *u, float *cvg,
                                                    int *itNum, float *seconds)
{
    return one_shot(ctx, opt, ASETS_BINARY, 3, Ny, Nx, Nz, 1, alpha, Cs, Ct, maxIt, errBound, cc,
                    steps, u, cvg, itNum, seconds);
}

extern "C" ASETS_API asets_status asets_potts2d(asets_context *ctx, const asets_options *opt,
                                                const float *alpha, const float *Ct, int Nx,
                                                int Ny, int nLab, int maxIt, float errBound,
                                                float cc, float steps, float *u, float *cvg,
                                                int *itNum, float *seconds)
{
    return one_shot(ctx, opt, ASETS_POTTS, 2, Ny, Nx, 1, nLab, alpha, nullptr, Ct, maxIt,
                    errBound, cc, steps, u, cvg, itNum, seconds);
}

extern "C" ASETS_API asets_status asets_potts3d(asets_context *ctx, const asets_options *opt,
                                                const float *alpha, const float *Ct, int Nx,
                                                int Ny, int Nz, int nLab, int maxIt,
                                                float errBound, float cc, float steps, float *u,
                                                float *cvg, int *itNum, float *seconds)
{
    return one_shot(ctx, opt, ASETS_POTTS, 3, Ny, Nx, Nz, nLab, alpha, nullptr, Ct, maxIt,
                    errBound, cc, steps, u, cvg, itNum, seconds);
}

extern "C" ASETS_API asets_status asets_ishikawa2d(asets_context *ctx, const asets_options *opt,
                                                   const float *alpha, const float *Ct, int Nx,
                                                   int Ny, int nLab, int maxIt, float errBound,
                                                   float cc, float steps, float *u, float *cvg,
                                                   int *itNum, float *seconds)
{
    return one_shot(ctx, opt, ASETS_ISHIKAWA, 2, Ny, Nx, 1, nLab, alpha, nullptr, Ct, maxIt,
                    errBound, cc, steps, u, cvg, itNum, seconds);
}

extern "C" ASETS_API asets_status asets_ishikawa3d(asets_context *ctx, const asets_options *opt,
                                                   const float *alpha, const float *Ct, int Nx,
                                                   int Ny, int Nz, int nLab, int maxIt,
                                                   float errBound, float cc, float steps,
                                                   float *u, float *cvg, int *itNum,
                                                   float *seconds)
{
    return one_shot(ctx, opt, ASETS_ISHIKAWA, 3, Ny, Nx, Nz, nLab, alpha, nullptr, Ct, maxIt,
                    errBound, cc, steps, u, cvg, itNum, seconds);
}
