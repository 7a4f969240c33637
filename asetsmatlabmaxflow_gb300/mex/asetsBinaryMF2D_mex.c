/*
 * GPU drop-in for maxflow/asetsBinaryMF2D_mex.c:36-129:
 *   [u, erriter, i, timet] = asetsBinaryMF2D_mex(single ...inputs..., single pars)
 * Build with Matlab: mex -compatibleArrayDims asetsBinaryMF2D_mex.c -L<lib> -lasetscuda
 */
#include "asets_mex_common.h"

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    asets_mex_run(MEX_BINARY, 2, nlhs, plhs, nrhs, prhs, "binary max flow 2D");
}
