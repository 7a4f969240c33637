// Host-side set-up of the fused iteration kernel: TMA descriptors for the
// halo and tile boxes of both ping-pong parities, destinations, work split.
#include <cstring>

#include "internal.h"

namespace asets {

static int encode(EncodeTiledFn fn, CUtensorMap *map, float *base, const StencilProblem &p,
                  int labels, int box_rows, int box_cols, int box_labels = 1)
{
    cuuint64_t dims[4] = {(cuuint64_t)p.nr, (cuuint64_t)p.nc, (cuuint64_t)p.ns,
                          (cuuint64_t)(labels < 1 ? 1 : labels)};
    cuuint64_t strides[3] = {(cuuint64_t)(p.pitch * 4), (cuuint64_t)(p.plane * 4),
                             (cuuint64_t)(p.cells * 4)};
    cuuint32_t box[4] = {(cuuint32_t)box_rows, (cuuint32_t)box_cols, 1, (cuuint32_t)box_labels};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return (int)r;
}

int build_problem_desc(EncodeTiledFn fn, const StencilVariant &v, const StencilProblem &p,
                       ProblemDesc *A)
{
    memset(A, 0, sizeof *A);
    const bool binary = (v.epi == EPI_BINARY);
    // label extent of each slot's box
    auto box_labels = [&](int labels) { return v.label_boxes == LB_ALL ? labels : 1; };
    for (int par = 0; par < 2; ++par) {
        float *srcs[NUM_SLOTS] = {p.b[par][0], p.b[par][1], p.b[par][2], p.src[par][0],
                                  p.src[par][1], p.src[par][2], p.alpha};
        int labels[NUM_SLOTS] = {p.flow_labels, p.flow_labels, p.flow_labels, p.src_labels[0],
                                 p.src_labels[1], p.src_labels[2], p.alpha_labels};
        for (int slot = 0; slot < NUM_SLOTS; ++slot) {
            if (v.dim == 2 && slot == SL_BC)
                continue;
            const int cols = (slot == SL_BC) ? v.box_cols_bc : v.box_cols;
            int r = encode(fn, &A->halo[par][slot], srcs[slot], p, labels[slot], v.box_rows, cols,
                           box_labels(labels[slot]));
            if (r)
                return r;
        }
        if (binary) {
            float *tsrc[NUM_TILE_SLOTS] = {p.src[par][1], p.src[par][2], const_cast<float *>(p.cs),
                                           const_cast<float *>(p.ct)};
            for (int ts = 0; ts < NUM_TILE_SLOTS; ++ts) {
                int r = encode(fn, &A->tile[par][ts], tsrc[ts], p, 1,
                               v.tile_box_rows > 0 ? v.tile_box_rows : v.tr, v.tc);
                if (r)
                    return r;
            }
        }
        if (v.ct_box_rows > 0) {
            int r = encode(fn, &A->tile[par][TS_CT], const_cast<float *>(p.ct), p, p.ct_labels,
                           v.ct_box_rows, v.box_cols, box_labels(p.ct_labels));
            if (r)
                return r;
        }
        for (int k = 0; k < 3; ++k) {
            A->dst_b[par][k] = p.b[par ^ 1][k];
            A->dst_s[par][k] = p.dst_s[par][k];
        }
    }
    for (int s = 0; s < NUM_SLOTS; ++s) {
        A->lab_mul[s] = p.lab_mul[s];
        A->lab_add[s] = p.lab_add[s];
    }
    A->alpha = p.alpha;
    A->cs = p.cs;
    A->ct = p.ct;
    A->pitch = p.pitch;
    // the largest destination: the flows, or the new pt of a one-pass
    // multi-label kernel (Ishikawa: one label more than the flows)
    A->dst_elems = p.cells * (p.flow_labels > 0 ? p.flow_labels : 1);
    if (v.ct_box_rows > 0 && p.ct_labels > p.flow_labels)
        A->dst_elems = p.cells * p.ct_labels;
    A->plane_stride = p.plane;
    A->label_stride = p.cells;
    A->nr = p.nr;
    A->nc = p.nc;
    A->ns = p.ns;
    A->nlab_items = p.flow_labels;
    A->tiles_r = (p.nr + v.tr - 1) / v.tr;
    A->tiles_c = (v.dim == 3) ? (p.nc + v.tc - 1) / v.tc : 1;
    A->zchunks = 1;
    return 0;
}

// labels swept by one item: one, or all of them in the one-pass kernel
static int item_labels(const StencilProblem &p, const StencilVariant &v)
{
    return v.epi == EPI_FUSED ? 1 : p.flow_labels;
}

int problem_items(const StencilProblem &p, const StencilVariant &v, int zchunks)
{
    const long long tiles = (long long)((p.nr + v.tr - 1) / v.tr) *
                            ((v.dim == 3) ? (p.nc + v.tc - 1) / v.tc : 1);
    return (int)(tiles * item_labels(p, v) * zchunks);
}

int choose_zchunks(const StencilProblem &p, const StencilVariant &v, long long slots)
{
    const long long tiles = (long long)((p.nr + v.tr - 1) / v.tr) *
                            ((v.dim == 3) ? (p.nc + v.tc - 1) / v.tc : 1) * item_labels(p, v);
    if (v.s_tile > 0)
        return (p.ns + v.s_tile - 1) / v.s_tile;  // square tiles: one item per tile
    if (slots < 1 || tiles < 1)
        return 1;
    // Items (tile, chunk) run in waves of `slots` blocks; each chunk pays a
    // 4-plane warm-up.  Pick the chunk count with the best
    // (wave fill) x (useful planes / swept planes), chunks >= 8 planes.
    const long long max_k = p.ns / 8 > 1 ? p.ns / 8 : 1;
    int best = 1;
    double best_eff = 0.0;
    for (long long k = 1; k <= max_k && k <= 64; ++k) {
        const long long items = tiles * k;
        const long long waves = (items + slots - 1) / slots;
        const double fill = (double)items / (double)(waves * slots);
        const double planes = (double)p.ns / (double)k;
        const double eff = fill * planes / (planes + 4.0);
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = (int)k;
        }
    }
    return best;
}

}  // namespace asets
