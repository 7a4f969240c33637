/*
 * Host-side boundary code under AddressSanitizer and UndefinedBehaviorSanitizer
 * (tests/test_host_sanitize.py builds and runs this with -fsanitize=...):
 * the six mex drop-ins (asetsmatlabmaxflow_gb300/mex/asets*_mex.c with their
 * shared body), the MEX host emulation (mexshim.c) and the C oracle, with
 * the GPU library replaced by a fake whose asets_* solvers answer from the
 * oracle -- so argument parsing, output creation, error unwinding and
 * status mapping run end to end on the CPU.  Exit code 0: every case gave
 * the expected result and the sanitizers reported nothing (they abort).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "asets.h"
#include "asets_oracle.h"
#include "mex.h"

/* ---- the fake libasetscuda: the oracle behind the C ABI's solvers */
static char g_err[256];
const char *asets_status_string(asets_status s)
{
    static const char *names[] = {"ok", "invalid argument", "alpha", "cuda", "out of memory",
                                  "timeout", "no device", "unsupported"};
    return (s >= 0 && s <= 7) ? names[s] : "?";
}
const char *asets_last_error(void) { return g_err; }

static asets_status fake(int model, int dim, const float *alpha, const float *cs,
                         const float *ct, int nx, int ny, int nz, int nlab, int max_it,
                         float eb, float cc, float steps, float *u, float *cvg, int *it_num,
                         float *seconds)
{
    oracle_problem p;
    memset(&p, 0, sizeof p);
    p.model = model;
    p.dim = dim;
    p.ny = ny;
    p.nx = nx;
    p.nz = nz;
    p.nlab = nlab;
    p.max_it = max_it;
    p.err_bound = eb;
    p.cc = cc;
    p.steps = steps;
    p.alpha = alpha;
    p.cs = cs;
    p.ct = ct;
    p.u = u;
    p.cvg = cvg;
    p.it_num = it_num;
    const int rc = oracle_solve(&p);
    if (seconds)
        *seconds = 0.001f;
    if (rc == 1)
        return ASETS_ERR_ALPHA;
    if (rc) {
        snprintf(g_err, sizeof g_err, "oracle code %d", rc);
        return ASETS_ERR_INVALID_ARG;
    }
    return ASETS_OK;
}

asets_status asets_binary_mf2d(asets_context *c, const asets_options *o, const float *alpha,
                               const float *Cs, const float *Ct, int Nx, int Ny, int maxIt,
                               float eb, float cc, float steps, float *u, float *cvg, int *it,
                               float *sec)
{
    (void)c, (void)o;
    return fake(ORACLE_BINARY, 2, alpha, Cs, Ct, Nx, Ny, 1, 1, maxIt, eb, cc, steps, u, cvg, it, sec);
}
asets_status asets_binary_mf3d(asets_context *c, const asets_options *o, const float *alpha,
                               const float *Cs, const float *Ct, int Nx, int Ny, int Nz, int maxIt,
                               float eb, float cc, float steps, float *u, float *cvg, int *it,
                               float *sec)
{
    (void)c, (void)o;
    return fake(ORACLE_BINARY, 3, alpha, Cs, Ct, Nx, Ny, Nz, 1, maxIt, eb, cc, steps, u, cvg, it,
                sec);
}
asets_status asets_potts2d(asets_context *c, const asets_options *o, const float *alpha,
                           const float *Ct, int Nx, int Ny, int L, int maxIt, float eb, float cc,
                           float steps, float *u, float *cvg, int *it, float *sec)
{
    (void)c, (void)o;
    return fake(ORACLE_POTTS, 2, alpha, NULL, Ct, Nx, Ny, 1, L, maxIt, eb, cc, steps, u, cvg, it, sec);
}
asets_status asets_potts3d(asets_context *c, const asets_options *o, const float *alpha,
                           const float *Ct, int Nx, int Ny, int Nz, int L, int maxIt, float eb,
                           float cc, float steps, float *u, float *cvg, int *it, float *sec)
{
    (void)c, (void)o;
    return fake(ORACLE_POTTS, 3, alpha, NULL, Ct, Nx, Ny, Nz, L, maxIt, eb, cc, steps, u, cvg, it,
                sec);
}
asets_status asets_ishikawa2d(asets_context *c, const asets_options *o, const float *alpha,
                              const float *Ct, int Nx, int Ny, int L, int maxIt, float eb, float cc,
                              float steps, float *u, float *cvg, int *it, float *sec)
{
    (void)c, (void)o;
    return fake(ORACLE_ISHIKAWA, 2, alpha, NULL, Ct, Nx, Ny, 1, L, maxIt, eb, cc, steps, u, cvg, it,
                sec);
}
asets_status asets_ishikawa3d(asets_context *c, const asets_options *o, const float *alpha,
                              const float *Ct, int Nx, int Ny, int Nz, int L, int maxIt, float eb,
                              float cc, float steps, float *u, float *cvg, int *it, float *sec)
{
    (void)c, (void)o;
    return fake(ORACLE_ISHIKAWA, 3, alpha, NULL, Ct, Nx, Ny, Nz, L, maxIt, eb, cc, steps, u, cvg,
                it, sec);
}

/* the six drop-ins, each compiled with -DmexFunction=mexFunction_<name> */
void mexFunction_b2(int, mxArray *[], int, const mxArray *[]);
void mexFunction_b3(int, mxArray *[], int, const mxArray *[]);
void mexFunction_p2(int, mxArray *[], int, const mxArray *[]);
void mexFunction_p3(int, mxArray *[], int, const mxArray *[]);
void mexFunction_i2(int, mxArray *[], int, const mxArray *[]);
void mexFunction_i3(int, mxArray *[], int, const mxArray *[]);

static unsigned g_seed = 12345u;
static float frand(void)
{
    g_seed = g_seed * 1664525u + 1013904223u;
    return (float)(g_seed >> 8) / 16777216.0f;
}

static mxArray *single_array(int nd, const int *dims, float lo, float hi)
{
    mxArray *a = mxCreateNumericArray(nd, dims, mxSINGLE_CLASS, mxREAL);
    float *p = (float *)mxGetData(a);
    for (size_t i = 0; i < mxGetNumberOfElements(a); ++i)
        p[i] = lo + (hi - lo) * frand();
    return a;
}

static int g_fail = 0;
#define CHECK(cond, ...)                          \
    do {                                          \
        if (!(cond)) {                            \
            fprintf(stderr, "FAIL: " __VA_ARGS__); \
            fputc('\n', stderr);                  \
            g_fail = 1;                           \
        }                                         \
    } while (0)

/* One call: model 0/1/2, dim 2/3; returns 0 (ok) or 1 (mexErrMsgTxt) and the message. */
static int run_case(int model, int dim, int ny, int nx, int nz, int L, int max_it, float eb,
                    float alpha_lo, int wrong_class, int nrhs_short, char *msg)
{
    mexshim_entry fns[3][2] = {{mexFunction_b2, mexFunction_b3},
                               {mexFunction_p2, mexFunction_p3},
                               {mexFunction_i2, mexFunction_i3}};
    int vd[4] = {ny, nx, nz, L};
    int nd = dim;
    int cdims[4] = {ny, nx, dim == 3 ? nz : L, L};
    const int la = model == 1 ? L : L - 1;
    int adims[4] = {ny, nx, dim == 3 ? nz : la, la};
    mxArray *in[4];
    int nin = 0;
    if (model == 0) {
        in[nin++] = single_array(nd, vd, 0.f, 1.f);
        in[nin++] = single_array(nd, vd, 0.f, 1.f);
        in[nin++] = single_array(nd, vd, alpha_lo, 0.6f);
    } else {
        in[nin++] = single_array(nd + 1, cdims, 0.f, 1.f);
        in[nin++] = single_array(nd + 1, adims, alpha_lo, 0.5f);
    }
    float pars[8];
    int np = 0;
    pars[np++] = (float)ny;
    pars[np++] = (float)nx;
    if (dim == 3)
        pars[np++] = (float)nz;
    if (model)
        pars[np++] = (float)L;
    pars[np++] = (float)max_it;
    pars[np++] = eb;
    pars[np++] = 0.3f;
    pars[np++] = dim == 3 ? 0.11f : 0.16f;
    int pd[2] = {np, 1};
    mxArray *pa = mxCreateNumericArray(2, pd, wrong_class ? mxDOUBLE_CLASS : mxSINGLE_CLASS, mxREAL);
    if (!wrong_class)
        memcpy(mxGetData(pa), pars, sizeof(float) * np);
    in[nin++] = pa;
    mxArray *out[4] = {NULL, NULL, NULL, NULL};
    const int rc = mexshim_call(fns[model][dim - 2], 4, out, nrhs_short ? nin - 1 : nin,
                                (const mxArray **)in, msg, 256);
    if (rc == 0) {
        /* outputs as the reference creates them */
        CHECK(out[0] && out[1] && out[2] && out[3], "missing outputs");
        CHECK(mxGetClassID(out[2]) == mxUINT16_CLASS, "itNum class");
        CHECK(mxGetNumberOfElements(out[1]) == (size_t)max_it, "cvg length");
        const uint16_t it = *(const uint16_t *)mxGetData(out[2]);
        CHECK((int)it <= max_it, "itNum %d > maxIt %d", (int)it, max_it);
        const float *u = (const float *)mxGetData(out[0]);
        for (size_t i = 0; i < mxGetNumberOfElements(out[0]); ++i)
            CHECK(isfinite(u[i]), "non-finite u");
        for (int i = 0; i < 4; ++i)
            mxDestroyArray(out[i]);
    }
    for (int i = 0; i < nin; ++i)
        mxDestroyArray(in[i]);
    return rc;
}

int main(void)
{
    char msg[256];
    for (int model = 0; model < 3; ++model) {
        for (int dim = 2; dim <= 3; ++dim) {
            const int L = model == 0 ? 1 : (model == 1 ? 3 : 4);
            /* regular solves, odd and degenerate shapes */
            const int shapes[][3] = {{17, 13, 5}, {1, 1, 1}, {1, 9, 3}, {23, 1, 2}};
            for (int s = 0; s < 4; ++s) {
                int rc = run_case(model, dim, shapes[s][0], shapes[s][1], shapes[s][2], L, 12, 1e-4f,
                                  0.1f, 0, 0, msg);
                CHECK(rc == 0, "model %d dim %d shape %d: %s", model, dim, s, msg);
            }
            /* maxIt = 0: no iteration, no alpha check */
            CHECK(run_case(model, dim, 9, 7, 3, L, 0, 0.f, -1.f, 0, 0, msg) == 0, "maxIt 0: %s", msg);
            /* alpha <= 0: the reference's message */
            int rc = run_case(model, dim, 9, 7, 3, L, 5, 0.f, -1.f, 0, 0, msg);
            CHECK(rc == 1 && strstr(msg, "must be positive"), "alpha error: %d %s", rc, msg);
            /* wrong class and missing input: a clean mexErrMsgTxt */
            rc = run_case(model, dim, 9, 7, 3, L, 5, 0.f, 0.1f, 1, 0, msg);
            CHECK(rc == 1 && strstr(msg, "single"), "class error: %d %s", rc, msg);
            rc = run_case(model, dim, 9, 7, 3, L, 5, 0.f, 0.1f, 0, 1, msg);
            CHECK(rc == 1 && strstr(msg, "expected inputs"), "nrhs error: %d %s", rc, msg);
        }
    }
    /* the shim's arrays of every class and of zero, one and many elements */
    const mxClassID cls[] = {mxDOUBLE_CLASS, mxSINGLE_CLASS, mxINT8_CLASS, mxUINT8_CLASS,
                             mxINT16_CLASS, mxUINT16_CLASS, mxINT32_CLASS, mxUINT32_CLASS};
    const int dd[][3] = {{0, 3, 1}, {1, 1, 1}, {5, 4, 3}};
    for (int c = 0; c < 8; ++c)
        for (int d = 0; d < 3; ++d) {
            mxArray *a = mxCreateNumericArray(3, dd[d], cls[c], mxREAL);
            CHECK(a != NULL, "create class %d", c);
            memset(mxGetData(a), 0, mxGetNumberOfElements(a) ? mxGetNumberOfElements(a) : 1);
            mxDestroyArray(a);
        }
    if (!g_fail)
        printf("sanitized host boundary: all cases ok\n");
    return g_fail;
}
