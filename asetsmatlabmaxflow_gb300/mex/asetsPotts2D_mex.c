/*
 * GPU drop-in for maxflow/asetsPotts2D_mex.c:42-135:
 *   [u, erriter, i, timet] = asetsPotts2D_mex(single ...inputs..., single pars)
 * Build with Matlab: mex -compatibleArrayDims asetsPotts2D_mex.c -L<lib> -lasetscuda
 */
#include "asets_mex_common.h"

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    asets_mex_run(MEX_POTTS, 2, nlhs, plhs, nrhs, prhs, "potts model max flow 2D");
}
