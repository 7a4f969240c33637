/*
 * Shared body of the six GPU mex entry points.
 *
 * Each reproduces its reference mexFunction (e.g. maxflow/asetsBinaryMF3D_mex.c:39-134):
 * same inputs (single Cs?, Ct, alpha, pars), same positional pars layout, the
 * same four outputs [u, erriter, i, timet] created regardless of nlhs, the
 * same error text for alpha <= 0 and the same progress line.  Two reference
 * defects are not reproduced: `i` is written as a real uint16 (the reference
 * stores a 4-byte int into it) and `timet` as a real single holding the wall
 * seconds of the call (the reference stores a double's bytes into it).
 * Inputs are checked for count and class, where the reference would read
 * past the arrays.
 */
#ifndef ASETS_MEX_COMMON_H
#define ASETS_MEX_COMMON_H

#include <stdint.h>
#include <stdio.h>

#include "asets.h"
#include "mex.h"

enum { MEX_BINARY = 0, MEX_POTTS = 1, MEX_ISHIKAWA = 2 };

static void asets_mex_check_single(const mxArray *a, const char *what)
{
    char msg[160];
    if (!a || mxGetClassID(a) != mxSINGLE_CLASS) {
        snprintf(msg, sizeof msg, "%s must be a single (float32) array", what);
        mexErrMsgTxt(msg);
    }
}

static void asets_mex_run(int model, int dim, int nlhs, mxArray *plhs[], int nrhs,
                          const mxArray *prhs[], const char *banner)
{
    (void)nlhs;
    const int nin = (model == MEX_BINARY) ? 4 : 3;
    if (nrhs < nin)
        mexErrMsgTxt(model == MEX_BINARY ? "expected inputs (Cs, Ct, alpha, pars)"
                                         : "expected inputs (Ct, alpha, pars)");
    const mxArray *mCs = (model == MEX_BINARY) ? prhs[0] : NULL;
    const mxArray *mCt = prhs[nin - 3];
    const mxArray *mAl = prhs[nin - 2];
    const mxArray *mPa = prhs[nin - 1];
    if (mCs)
        asets_mex_check_single(mCs, "Cs");
    asets_mex_check_single(mCt, "Ct");
    asets_mex_check_single(mAl, "alpha");
    asets_mex_check_single(mPa, "pars");
    const float *pars = (const float *)mxGetData(mPa);
    /* pars: [rows, cols, (slices), (labels), maxIt, errBound, cc, steps] */
    const size_t npars = mxGetNumberOfElements(mPa);
    const size_t need = (size_t)(dim + (model == MEX_BINARY ? 0 : 1) + 4);
    if (npars < need)
        mexErrMsgTxt("pars has too few entries");
    int p = 0;
    const int Ny = (int)pars[p++];
    const int Nx = (int)pars[p++];
    const int Nz = (dim == 3) ? (int)pars[p++] : 1;
    const int nLab = (model == MEX_BINARY) ? 1 : (int)pars[p++];
    const int maxIt = (int)pars[p++];
    const float errBound = (float)pars[p++];
    const float cc = (float)pars[p++];
    const float steps = (float)pars[p++];
    if (Ny < 1 || Nx < 1 || Nz < 1 || maxIt < 0)
        mexErrMsgTxt("pars: sizes must be positive and maxIt non-negative");
    const size_t n = (size_t)Ny * Nx * Nz;
    const size_t nct = (model == MEX_BINARY) ? n : n * (size_t)nLab;
    const size_t nal = (model == MEX_BINARY) ? n : n * (size_t)(model == MEX_POTTS ? nLab : nLab - 1);
    if (mxGetNumberOfElements(mCt) < nct || mxGetNumberOfElements(mAl) < nal ||
        (mCs && mxGetNumberOfElements(mCs) < n))
        mexErrMsgTxt("input arrays are smaller than pars says");

    /* outputs, shaped as in the reference (e.g. asetsPotts3D_mex.c:95-123) */
    int dims[4];
    int nd = 0;
    dims[nd++] = Ny;
    dims[nd++] = Nx;
    if (dim == 3)
        dims[nd++] = Nz;
    if (model == MEX_POTTS)
        dims[nd++] = nLab;
    else if (model == MEX_ISHIKAWA)
        dims[nd++] = nLab - 1;
    plhs[0] = mxCreateNumericArray(nd, dims, mxSINGLE_CLASS, mxREAL);
    int d2[2] = {maxIt, 1};
    plhs[1] = mxCreateNumericArray(2, d2, mxSINGLE_CLASS, mxREAL);
    int d1[2] = {1, 1};
    plhs[2] = mxCreateNumericArray(2, d1, mxUINT16_CLASS, mxREAL);
    plhs[3] = mxCreateNumericArray(2, d1, mxSINGLE_CLASS, mxREAL);
    float *u = (float *)mxGetData(plhs[0]);
    float *cvg = (float *)mxGetData(plhs[1]);
    uint16_t *it_out = (uint16_t *)mxGetData(plhs[2]);
    float *timet = (float *)mxGetData(plhs[3]);

    const float *Cs = mCs ? (const float *)mxGetData(mCs) : NULL;
    const float *Ct = (const float *)mxGetData(mCt);
    const float *alpha = (const float *)mxGetData(mAl);
    int itNum = 0;
    float secs = 0.f;
    asets_status st;
    if (model == MEX_BINARY && dim == 2)
        st = asets_binary_mf2d(NULL, NULL, alpha, Cs, Ct, Nx, Ny, maxIt, errBound, cc, steps, u,
                               cvg, &itNum, &secs);
    else if (model == MEX_BINARY)
        st = asets_binary_mf3d(NULL, NULL, alpha, Cs, Ct, Nx, Ny, Nz, maxIt, errBound, cc, steps,
                               u, cvg, &itNum, &secs);
    else if (model == MEX_POTTS && dim == 2)
        st = asets_potts2d(NULL, NULL, alpha, Ct, Nx, Ny, nLab, maxIt, errBound, cc, steps, u, cvg,
                           &itNum, &secs);
    else if (model == MEX_POTTS)
        st = asets_potts3d(NULL, NULL, alpha, Ct, Nx, Ny, Nz, nLab, maxIt, errBound, cc, steps, u,
                           cvg, &itNum, &secs);
    else if (dim == 2)
        st = asets_ishikawa2d(NULL, NULL, alpha, Ct, Nx, Ny, nLab, maxIt, errBound, cc, steps, u,
                              cvg, &itNum, &secs);
    else
        st = asets_ishikawa3d(NULL, NULL, alpha, Ct, Nx, Ny, Nz, nLab, maxIt, errBound, cc, steps,
                              u, cvg, &itNum, &secs);
    if (st == ASETS_ERR_ALPHA)
        mexErrMsgTxt(model == MEX_BINARY ? "alpha(x) must be positive. Exiting..."
                                         : "alpha(x,l) must be positive. Exiting...");
    if (st != ASETS_OK) {
        char msg[600];
        snprintf(msg, sizeof msg, "libasetscuda: %s (%s)", asets_status_string(st),
                 asets_last_error());
        mexErrMsgTxt(msg);
    }
    *it_out = (uint16_t)itNum;
    *timet = secs;
    mexPrintf("%s: number of iterations = %i; time = %.4f sec\n", banner, itNum, (double)secs);
}

#endif
