/*
 * GPU drop-in for maxflow/asetsPotts3D_mex.c:44-141:
 *   [u, erriter, i, timet] = asetsPotts3D_mex(single ...inputs..., single pars)
 * Build with Matlab: mex -compatibleArrayDims asetsPotts3D_mex.c -L<lib> -lasetscuda
 */
#include "asets_mex_common.h"

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    asets_mex_run(MEX_POTTS, 3, nlhs, plhs, nrhs, prhs, "potts model max flow 3D");
}
