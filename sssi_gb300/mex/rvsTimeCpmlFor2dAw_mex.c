/*
 * rvsTimeCpmlFor2dAw_mex.c -- MEX gateway of 2D acoustic reverse propagation
 * on the GPU.  Drop-in replacement for src/fd_cmex/rvsTimeCpmlFor2dAw_mex.c:38-287.
 *
 *   [model, snapshot] = rvsTimeCpmlFor2dAw_mex(v, data, nDiffOrder, nBoundary, dz, dx, dt)
 *     v        nz x nx                velocity (already padded by extBoundary)
 *     data     nx x nt                surface data, injected on the top interior row, t = nt..1
 *     model    (nz+2l) x (nx+2l)      padded field one step before the last one computed
 *                                     (what the reference returns), l = 2*nDiffOrder-1
 *     snapshot nz x nx x nt           interior field of every step
 *
 * Arithmetic as in fwdTimeCpmlFor2dAw_mex.c (SSSI_MEX_MODE).
 */
#include <stdlib.h>
#include <string.h>

#include "mex.h"
#include "sssi_gb300.h"

static int sssi_mex_mode(void) {
    const char *m = getenv("SSSI_MEX_MODE");
    if (m && !strcmp(m, "strict")) return SSSI_MODE_FP64_STRICT;
    if (m && !strcmp(m, "fp32")) return SSSI_MODE_FP32;
    return SSSI_MODE_FP64;
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    mwSize nz, nx, nt, snapdims[3];
    int order, boundary, l, rc;
    (void)nlhs;

    if (nrhs < 7) mexErrMsgTxt("All 7 input arguments shall be provided!");

    nz = mxGetM(prhs[0]);
    nx = mxGetN(prhs[0]);
    if (mxGetM(prhs[1]) != nx) mexErrMsgTxt("Velocity model and input data should have the same x-axis grids!");
    nt = mxGetN(prhs[1]);
    order = (int)*mxGetPr(prhs[2]);
    boundary = (int)*mxGetPr(prhs[3]);
    l = 2 * order - 1;
    if (order < 1) mexErrMsgTxt("nDiffOrder must be positive!");

    snapdims[0] = nz;
    snapdims[1] = nx;
    snapdims[2] = nt;
    plhs[1] = mxCreateNumericArray(3, snapdims, mxDOUBLE_CLASS, mxREAL);
    plhs[0] = mxCreateDoubleMatrix(nz + 2 * (mwSize)l, nx + 2 * (mwSize)l, mxREAL);

    rc = sssi_rvsTimeCpmlFor2dAw(mxGetPr(prhs[0]), mxGetPr(prhs[1]), (int64_t)nz, (int64_t)nx, (int64_t)nt, order,
                                 boundary, *mxGetPr(prhs[4]), *mxGetPr(prhs[5]), *mxGetPr(prhs[6]),
                                 mxGetPr(plhs[0]), mxGetPr(plhs[1]), sssi_mex_mode());
    if (rc != SSSI_OK) mexErrMsgIdAndTxt("sssi:rvsTimeCpmlFor2dAw", "%s", sssi_last_error());
}
