/*
 * ORACLE -- test infrastructure only (the checker and the timed CPU
 * baseline); the product never links or calls this file.
 *
 * Restatement of the augmented-Lagrangian continuous max-flow iteration of
 * ASETS' six C mex solvers:
 *   binary    maxflow/asetsBinaryMF2D_mex.c:132-358, asetsBinaryMF3D_mex.c:137-438
 *   Potts     maxflow/asetsPotts2D_mex.c:138-434,   asetsPotts3D_mex.c:144-521
 *   Ishikawa  maxflow/asetsIshikawa2D_mex.c:136-482, asetsIshikawa3D_mex.c:141-610
 *
 * Storage differs from the reference: each flow component is kept per cell
 * (the face between a cell and its lower neighbour along that axis), the
 * faces on the lower domain border are never written and stay zero, and a
 * forward face beyond the upper border reads as zero.  The reference gets
 * the same zero-flux border by reading never-written entries of its
 * (N+1)-sized face arrays.  The floating-point expressions keep the
 * reference's operation order and precision (float everywhere, |p| in
 * double) so that results are bit-identical when both are compiled without
 * FMA contraction (-ffp-contract=off).
 */
#include "asets_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int dim, ny, nx, nz;
    size_t n;     /* cells */
    size_t plane; /* ny * nx */
} grid_t;

/* MIN/ABS exactly as the reference macros (asetsBinaryMF2D_mex.c:17-19):
 * the NaN behaviour of `a < b ? a : b` differs from fminf. */
static inline float min_ref(float a, float b) { return (a < b) ? a : b; }
static inline float abs_ref(float x) { return (x > 0.0) ? x : -x; }

/* One label's spatial-flow update: updateP1, updatePX/PY/PZ, projStep,
 * updateBX/BY/BZ and the divergence (asetsBinaryMF3D_mex.c:226-416).
 * The gk source term is (s0 - s1) + s2/cc:
 *   binary  (ps, pt, u)         asetsBinaryMF3D_mex.c:238
 *   Potts   (ps, pt_k, u_k)     asetsPotts3D_mex.c:273
 *   Ishikawa(pt_k, pt_k+1, u_k) asetsIshikawa3D_mex.c:287
 * dv holds div(b) of the previous iteration on entry and of the new flow on
 * return.  Returns nonzero if some alpha <= 0 (projStep's check). */
static int flow_update(const grid_t *g, float *bx, float *by, float *bz,
                       float *dv, float *gk, const float *alpha,
                       const float *s0, const float *s1, const float *s2,
                       float cc, float steps)
{
    const int ny = g->ny, nx = g->nx, nz = g->nz;
    const size_t pl = g->plane;
    const int three = (g->dim == 3);

    /* gk = dv - (s0 - s1 + s2/cc) */
    for (size_t c = 0; c < g->n; ++c)
        gk[c] = dv[c] - (s0[c] - s1[c] + s2[c] / cc);

    /* projected-gradient step on interior faces */
    for (int z = 0; z < nz; ++z)
        for (int x = 0; x < nx; ++x) {
            size_t row = (size_t)z * pl + (size_t)x * ny;
            if (x >= 1)
                for (int y = 0; y < ny; ++y)
                    bx[row + y] = steps * (gk[row + y] - gk[row + y - ny]) + bx[row + y];
            for (int y = 1; y < ny; ++y)
                by[row + y] = steps * (gk[row + y] - gk[row + y - 1]) + by[row + y];
            if (three && z >= 1)
                for (int y = 0; y < ny; ++y)
                    bz[row + y] = steps * (gk[row + y] - gk[row + y - pl]) + bz[row + y];
        }

    /* projection |p(x)| <= alpha(x): the norm is formed in double */
    for (int z = 0; z < nz; ++z)
        for (int x = 0; x < nx; ++x) {
            size_t row = (size_t)z * pl + (size_t)x * ny;
            const int xlast = (x + 1 == nx), zlast = (z + 1 == nz);
            for (int y = 0; y < ny; ++y) {
                size_t c = row + y;
                float a = alpha[c];
                if (a <= 0)
                    return 1;
                double bx1 = xlast ? 0.0 : (double)bx[c + ny];
                double bx0 = bx[c];
                double by1 = (y + 1 == ny) ? 0.0 : (double)by[c + 1];
                double by0 = by[c];
                double s = bx1 * bx1 + bx0 * bx0 + by1 * by1 + by0 * by0;
                if (three) {
                    double bz1 = zlast ? 0.0 : (double)bz[c + pl];
                    double bz0 = bz[c];
                    s = s + bz1 * bz1 + bz0 * bz0;
                }
                float fpt = (float)sqrt(s * 0.5);
                if (fpt > a)
                    fpt = fpt / a;
                else
                    fpt = 1;
                gk[c] = 1 / fpt;
            }
        }

    /* rescale the interior faces by the mean of the two cells' factors */
    for (int z = 0; z < nz; ++z)
        for (int x = 0; x < nx; ++x) {
            size_t row = (size_t)z * pl + (size_t)x * ny;
            if (x >= 1)
                for (int y = 0; y < ny; ++y)
                    bx[row + y] = (float)((gk[row + y] + gk[row + y - ny]) * 0.5 * bx[row + y]);
            for (int y = 1; y < ny; ++y)
                by[row + y] = (float)(0.5 * (gk[row + y - 1] + gk[row + y]) * by[row + y]);
            if (three && z >= 1)
                for (int y = 0; y < ny; ++y)
                    bz[row + y] = (float)(0.5 * (gk[row + y - pl] + gk[row + y]) * bz[row + y]);
        }

    /* divergence of the new flow */
    for (int z = 0; z < nz; ++z)
        for (int x = 0; x < nx; ++x) {
            size_t row = (size_t)z * pl + (size_t)x * ny;
            const int xlast = (x + 1 == nx), zlast = (z + 1 == nz);
            for (int y = 0; y < ny; ++y) {
                size_t c = row + y;
                float by1 = (y + 1 == ny) ? 0.0f : by[c + 1];
                float bx1 = xlast ? 0.0f : bx[c + ny];
                float d = by1 - by[c] + bx1 - bx[c];
                if (three) {
                    float bz1 = zlast ? 0.0f : bz[c + pl];
                    d = d + bz1 - bz[c];
                }
                dv[c] = d;
            }
        }
    return 0;
}

/* First index of the minimum of Ct over labels, from a start of 1e30 /
 * 1e9 exactly as init() does (asetsPotts3D_mex.c:229-241). */
static void argmin_labels(const float *ct, size_t n, size_t c, int nlab,
                          float *min_val, int *min_id)
{
    float mv = 1e30f;
    int mi = 1000000000;
    for (int l = 0; l < nlab; ++l) {
        float v = ct[c + (size_t)l * n];
        if (mv > v) {
            mv = v;
            mi = l;
        }
    }
    *min_val = mv;
    *min_id = mi;
}

static int solve_binary(const oracle_problem *p, const grid_t *g)
{
    const size_t n = g->n;
    float *bx = calloc(n, sizeof(float)), *by = calloc(n, sizeof(float));
    float *bz = calloc(n, sizeof(float)), *dv = calloc(n, sizeof(float));
    float *gk = calloc(n, sizeof(float)), *ps = calloc(n, sizeof(float));
    float *pt = calloc(n, sizeof(float));
    float *u = p->u;
    int rc = ORACLE_OK;
    if (!bx || !by || !bz || !dv || !gk || !ps || !pt) {
        rc = ORACLE_ERR_NOMEM;
        goto done;
    }
    if (p->u0) {
        memcpy(u, p->u0, n * sizeof(float));
        memcpy(ps, p->ps0, n * sizeof(float));
        memcpy(pt, p->pt0, n * sizeof(float));
    } else {
        /* init: asetsBinaryMF3D_mex.c:205-224 */
        for (size_t c = 0; c < n; ++c) {
            u[c] = (p->cs[c] - p->ct[c] >= 0) ? 1.0f : 0.0f;
            ps[c] = min_ref(p->cs[c], p->ct[c]);
            pt[c] = ps[c];
        }
    }
    const float cc = p->cc;
    int i;
    for (i = 0; i < p->max_it; ++i) {
        if (flow_update(g, bx, by, bz, dv, gk, p->alpha, ps, pt, u, cc, p->steps)) {
            rc = ORACLE_ERR_ALPHA;
            goto done;
        }
        /* source/sink flows and multiplier: asetsBinaryMF3D_mex.c:418-432 */
        float erru_f = 0;
        double erru_d = 0;
        for (size_t c = 0; c < n; ++c) {
            float fpt = pt[c] - u[c] / cc + dv[c] + 1 / cc;
            ps[c] = min_ref(fpt, p->cs[c]);
            fpt = ps[c] + u[c] / cc - dv[c];
            pt[c] = min_ref(fpt, p->ct[c]);
            fpt = cc * (pt[c] + dv[c] - ps[c]);
            if (p->erru_double)
                erru_d += abs_ref(fpt);
            else
                erru_f += abs_ref(fpt);
            u[c] -= fpt;
        }
        float total = p->erru_double ? (float)erru_d : erru_f;
        p->cvg[i] = total / (float)(g->ny * g->nx * g->nz);
        if (p->cvg[i] <= p->err_bound)
            break;
    }
    *p->it_num = i;
    if (p->ps_out) memcpy(p->ps_out, ps, n * sizeof(float));
    if (p->pt_out) memcpy(p->pt_out, pt, n * sizeof(float));
done:
    free(bx); free(by); free(bz); free(dv); free(gk); free(ps); free(pt);
    return rc;
}

static int solve_potts(const oracle_problem *p, const grid_t *g)
{
    const size_t n = g->n;
    const int L = p->nlab;
    const size_t nl = n * (size_t)L;
    float *bx = calloc(nl, sizeof(float)), *by = calloc(nl, sizeof(float));
    float *bz = calloc(nl, sizeof(float)), *dv = calloc(nl, sizeof(float));
    float *gk = calloc(n, sizeof(float)), *ps = calloc(n, sizeof(float));
    float *pt = calloc(nl, sizeof(float)), *ft = calloc((size_t)L, sizeof(float));
    float *u = p->u;
    int rc = ORACLE_OK;
    if (!bx || !by || !bz || !dv || !gk || !ps || !pt || !ft) {
        rc = ORACLE_ERR_NOMEM;
        goto done;
    }
    if (p->u0) {
        memcpy(u, p->u0, nl * sizeof(float));
        memcpy(ps, p->ps0, n * sizeof(float));
        memcpy(pt, p->pt0, nl * sizeof(float));
    } else {
        /* init: asetsPotts3D_mex.c:219-258 */
        memset(u, 0, nl * sizeof(float));
        for (size_t c = 0; c < n; ++c) {
            float mv;
            int mi;
            argmin_labels(p->ct, n, c, L, &mv, &mi);
            ps[c] = mv;
            for (int l = 0; l < L; ++l) {
                pt[c + (size_t)l * n] = mv;
                if (l == mi)
                    u[c + (size_t)l * n] = 1.0f;
            }
        }
    }
    const float cc = p->cc;
    int i;
    for (i = 0; i < p->max_it; ++i) {
        for (int k = 0; k < L; ++k) {
            size_t o = (size_t)k * n;
            if (flow_update(g, bx + o, by + o, bz + o, dv + o, gk, p->alpha + o,
                            ps, pt + o, u + o, cc, p->steps)) {
                rc = ORACLE_ERR_ALPHA;
                goto done;
            }
            /* sink flow of label k with the previous ps: asetsPotts3D_mex.c:461-466 */
            for (size_t c = 0; c < n; ++c) {
                float fpt = ps[c] + u[o + c] / cc - dv[o + c];
                pt[o + c] = (fpt < p->ct[o + c]) ? fpt : p->ct[o + c];
            }
        }
        /* shared source flow and multipliers: asetsPotts3D_mex.c:474-521 */
        float erru_f = 0;
        double erru_d = 0;
        for (size_t c = 0; c < n; ++c) {
            float fpt = 0;
            for (int l = 0; l < L; ++l) {
                size_t o = c + (size_t)l * n;
                ft[l] = dv[o] + pt[o];
                fpt += (ft[l] - u[o] / cc);
            }
            ps[c] = fpt / L + 1 / (cc * L);
            for (int l = 0; l < L; ++l) {
                size_t o = c + (size_t)l * n;
                fpt = cc * (ft[l] - ps[c]);
                u[o] -= fpt;
                if (p->erru_double)
                    erru_d += abs_ref(fpt);
                else
                    erru_f += abs_ref(fpt);
            }
        }
        float total = p->erru_double ? (float)erru_d : erru_f;
        p->cvg[i] = total / (float)(g->ny * g->nx * g->nz * L);
        if (p->cvg[i] <= p->err_bound)
            break;
    }
    *p->it_num = i;
    if (p->ps_out) memcpy(p->ps_out, ps, n * sizeof(float));
    if (p->pt_out) memcpy(p->pt_out, pt, nl * sizeof(float));
done:
    free(bx); free(by); free(bz); free(dv); free(gk); free(ps); free(pt); free(ft);
    return rc;
}

static int solve_ishikawa(const oracle_problem *p, const grid_t *g)
{
    const size_t n = g->n;
    const int L = p->nlab;
    const size_t nf = n * (size_t)(L - 1); /* flow layers */
    float *bx = calloc(nf, sizeof(float)), *by = calloc(nf, sizeof(float));
    float *bz = calloc(nf, sizeof(float)), *dv = calloc(nf, sizeof(float));
    float *gk = calloc(n, sizeof(float));
    float *pt = calloc(n * (size_t)L, sizeof(float));
    float *u = p->u;
    int rc = ORACLE_OK;
    if (!bx || !by || !bz || !dv || !gk || !pt) {
        rc = ORACLE_ERR_NOMEM;
        goto done;
    }
    if (p->u0) {
        memcpy(u, p->u0, nf * sizeof(float));
        memcpy(pt, p->pt0, n * (size_t)L * sizeof(float));
    } else {
        /* init: asetsIshikawa3D_mex.c:230-270; the top layer pt_{L-1} stays 0 */
        for (size_t c = 0; c < n; ++c) {
            float mv;
            int mi;
            argmin_labels(p->ct, n, c, L, &mv, &mi);
            for (int l = 0; l < L - 1; ++l) {
                pt[c + (size_t)l * n] = mv;
                u[c + (size_t)l * n] = (l >= mi) ? 0.0f : 1.0f;
            }
        }
    }
    const float cc = p->cc;
    int i;
    for (i = 0; i < p->max_it; ++i) {
        for (int k = 0; k < L - 1; ++k) {
            size_t o = (size_t)k * n;
            if (flow_update(g, bx + o, by + o, bz + o, dv + o, gk, p->alpha + o,
                            pt + o, pt + o + n, u + o, cc, p->steps)) {
                rc = ORACLE_ERR_ALPHA;
                goto done;
            }
        }
        /* sink-flow chain over the ordered labels, lowest first, each layer
         * using the already updated layer below (asetsIshikawa3D_mex.c:189-201,
         * :498-576) */
        for (int k = 0; k < L; ++k) {
            size_t o = (size_t)k * n;
            for (size_t c = 0; c < n; ++c) {
                float fpt;
                if (k == 0) {
                    fpt = dv[o + c] + pt[o + c + n] - u[o + c] / cc + 1 / cc;
                } else if (k < L - 1) {
                    fpt = -dv[o + c - n] + pt[o + c - n] + u[o + c - n] / cc;
                    fpt += dv[o + c] + pt[o + c + n] - u[o + c] / cc;
                    fpt /= 2.0f;
                } else {
                    fpt = -dv[o + c - n] + pt[o + c - n] + u[o + c - n] / cc;
                }
                pt[o + c] = min_ref(fpt, p->ct[o + c]);
            }
        }
        /* multipliers: asetsIshikawa3D_mex.c:578-610 */
        float erru_f = 0;
        double erru_d = 0;
        for (size_t c = 0; c < n; ++c)
            for (int l = 0; l < L - 1; ++l) {
                size_t o = c + (size_t)l * n;
                float fpt = cc * (dv[o] + pt[o + n] - pt[o]);
                u[o] -= fpt;
                if (p->erru_double)
                    erru_d += abs_ref(fpt);
                else
                    erru_f += abs_ref(fpt);
            }
        float total = p->erru_double ? (float)erru_d : erru_f;
        p->cvg[i] = total / (float)(g->ny * g->nx * g->nz * (L - 1));
        /* 2D breaks on '<' (asetsIshikawa2D_mex.c:205), 3D on '<='
         * (asetsIshikawa3D_mex.c:213) */
        if (g->dim == 2 ? (p->cvg[i] < p->err_bound) : (p->cvg[i] <= p->err_bound))
            break;
    }
    *p->it_num = i;
    if (p->pt_out) memcpy(p->pt_out, pt, n * (size_t)L * sizeof(float));
done:
    free(bx); free(by); free(bz); free(dv); free(gk); free(pt);
    return rc;
}

int oracle_solve(const oracle_problem *p)
{
    if (!p || (p->dim != 2 && p->dim != 3) || p->ny < 1 || p->nx < 1 || p->nz < 1 ||
        p->max_it < 0 || !p->alpha || !p->ct || !p->u || !p->it_num ||
        (p->max_it > 0 && !p->cvg))
        return ORACLE_ERR_ARG;
    if (p->dim == 2 && p->nz != 1)
        return ORACLE_ERR_ARG;
    grid_t g;
    g.dim = p->dim;
    g.ny = p->ny;
    g.nx = p->nx;
    g.nz = p->nz;
    g.plane = (size_t)p->ny * (size_t)p->nx;
    g.n = g.plane * (size_t)p->nz;
    if (p->max_it > 0)
        memset(p->cvg, 0, (size_t)p->max_it * sizeof(float));
    switch (p->model) {
    case ORACLE_BINARY:
        if (!p->cs || (p->u0 && (!p->ps0 || !p->pt0)))
            return ORACLE_ERR_ARG;
        return solve_binary(p, &g);
    case ORACLE_POTTS:
        if (p->nlab < 1 || (p->u0 && (!p->ps0 || !p->pt0)))
            return ORACLE_ERR_ARG;
        return solve_potts(p, &g);
    case ORACLE_ISHIKAWA:
        if (p->nlab < 2 || (p->u0 && !p->pt0))
            return ORACLE_ERR_ARG;
        return solve_ishikawa(p, &g);
    default:
        return ORACLE_ERR_ARG;
    }
}
