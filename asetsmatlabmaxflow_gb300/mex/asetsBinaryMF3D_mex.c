/*
 * GPU drop-in for maxflow/asetsBinaryMF3D_mex.c:39-134:
 *   [u, erriter, i, timet] = asetsBinaryMF3D_mex(single ...inputs..., single pars)
 * Build with Matlab: mex -compatibleArrayDims asetsBinaryMF3D_mex.c -L<lib> -lasetscuda
 */
#include "asets_mex_common.h"

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    asets_mex_run(MEX_BINARY, 3, nlhs, plhs, nrhs, prhs, "binary max flow 3D");
}
