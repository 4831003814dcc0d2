/*
 * fwdTimeCpmlFor2dAw_mex.c -- MEX gateway of 2D acoustic forward modelling on
 * the GPU.  Drop-in replacement for src/fd_cmex/fwdTimeCpmlFor2dAw_mex.c:39-290:
 * same symbol, same inputs and outputs, so src/fd_cmex/fwdTimeCpmlFor2dAw.m and
 * every application script that calls it run unchanged.
 *
 *   [data, snapshot] = fwdTimeCpmlFor2dAw_mex(v, source, nDiffOrder, nBoundary, dz, dx, dt)
 *     v        nz x nx            velocity (already padded by extBoundary)
 *     source   nz x nx x nt       dense source
 *     data     nx x nt            top interior row of every step
 *     snapshot nz x nx x nt       interior field of every step
 *
 * The work is done by sssi_fwdTimeCpmlFor2dAw (libsssi_gb300).  Arithmetic:
 * fused FP64 (the batched tiled kernel; within 1e-12 relative L2 of the
 * reference) unless the environment variable SSSI_MEX_MODE is "strict" (FP64
 * with the reference's rounding sequence: bit-identical results, on a slower
 * row-marching kernel) or "fp32".
 *
 * Build against MATLAB:  mex -I<repo>/include fwdTimeCpmlFor2dAw_mex.c -L<lib> -lsssi_gb300
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
    const mwSize *dims;
    mwSize nd, nz, nx, nt, snapdims[3];
    int order, boundary, rc;
    (void)nlhs;

    if (nrhs < 7) mexErrMsgTxt("All 7 input arguments shall be provided!");

    dims = mxGetDimensions(prhs[1]);
    nd = mxGetNumberOfDimensions(prhs[1]);
    nz = dims[0];
    nx = dims[1];
    nt = nd >= 3 ? dims[2] : 1;
    if (mxGetM(prhs[0]) != nz || mxGetN(prhs[0]) != nx)
        mexErrMsgTxt("Velocity model and source grids should have the same z-axis and x-axis grids!");
    order = (int)*mxGetPr(prhs[2]);
    boundary = (int)*mxGetPr(prhs[3]);

    /* outputs always exist, as in the reference (even when nlhs < 2) */
    plhs[0] = mxCreateDoubleMatrix(nx, nt, mxREAL);
    snapdims[0] = nz;
    snapdims[1] = nx;
    snapdims[2] = nt;
    plhs[1] = mxCreateNumericArray(3, snapdims, mxDOUBLE_CLASS, mxREAL);

    rc = sssi_fwdTimeCpmlFor2dAw(mxGetPr(prhs[0]), mxGetPr(prhs[1]), (int64_t)nz, (int64_t)nx, (int64_t)nt, order,
                                 boundary, *mxGetPr(prhs[4]), *mxGetPr(prhs[5]), *mxGetPr(prhs[6]),
                                 mxGetPr(plhs[0]), mxGetPr(plhs[1]), sssi_mex_mode());
    if (rc != SSSI_OK) mexErrMsgIdAndTxt("sssi:fwdTimeCpmlFor2dAw", "%s", sssi_last_error());
}
