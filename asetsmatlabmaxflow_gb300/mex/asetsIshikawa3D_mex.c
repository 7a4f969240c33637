/*
 * GPU drop-in for maxflow/asetsIshikawa3D_mex.c:42-138:
 *   [u, erriter, i, timet] = asetsIshikawa3D_mex(single ...inputs..., single pars)
 * Build with Matlab: mex -compatibleArrayDims asetsIshikawa3D_mex.c -L<lib> -lasetscuda
 */
#include "asets_mex_common.h"

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    asets_mex_run(MEX_ISHIKAWA, 3, nlhs, plhs, nrhs, prhs, "ishikawa model max flow 3D");
}
