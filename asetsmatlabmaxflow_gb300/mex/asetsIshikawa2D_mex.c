/*
 * GPU drop-in for maxflow/asetsIshikawa2D_mex.c:40-133:
 *   [u, erriter, i, timet] = asetsIshikawa2D_mex(single ...inputs..., single pars)
 * Build with Matlab: mex -compatibleArrayDims asetsIshikawa2D_mex.c -L<lib> -lasetscuda
 */
#include "asets_mex_common.h"

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    asets_mex_run(MEX_ISHIKAWA, 2, nlhs, plhs, nrhs, prhs, "ishikawa model max flow 2D");
}
