/*
 * rvsTimeSpongeFor2dAw_mex.c -- MEX gateway of 2D acoustic reverse
 * propagation with the sponge absorbing boundary on the GPU.  The reference
 * computes this in MATLAB only (src/rvsTimeSpongeFor2dAw.m:1-103); with this
 * gateway that file becomes a one-line wrapper:
 *
 *   function [model, snapshot] = rvsTimeSpongeFor2dAw(v, data, nBoundary, dz, dx, dt)
 *   [model, snapshot] = rvsTimeSpongeFor2dAw_mex(v, data, nBoundary, dz, dx, dt);
 *
 *     v        nz x nx         velocity
 *     data     nx x nt         recorded data, entered on the top row with time
 *                              running backwards
 *     model    nz x nx         the field after the last step (the MATLAB file
 *                              declares this output and never assigns it)
 *     snapshot nz x nx x nt    field of every step (only computed when the
 *                              caller asks for two outputs)
 *
 * The work is done by sssi_rvsTimeSpongeFor2dAw (libsssi_gb300) in fused FP64
 * unless the environment variable SSSI_MEX_MODE is "strict" or "fp32".
 *
 * Build against MATLAB:  mex -I<repo>/include rvsTimeSpongeFor2dAw_mex.c -L<lib> -lsssi_gb300
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
    int boundary, rc;
    double *snap = NULL;

    if (nrhs < 6) mexErrMsgTxt("All 6 input arguments shall be provided!");

    nz = mxGetM(prhs[0]);
    nx = mxGetN(prhs[0]);
    nt = mxGetN(prhs[1]);
    if (mxGetM(prhs[1]) != nx) mexErrMsgTxt("Velocity model and data should have the same x-axis grids!");
    boundary = (int)*mxGetPr(prhs[2]);

    plhs[0] = mxCreateDoubleMatrix(nz, nx, mxREAL);
    if (nlhs >= 2) {
        snapdims[0] = nz;
        snapdims[1] = nx;
        snapdims[2] = nt;
        plhs[1] = mxCreateNumericArray(3, snapdims, mxDOUBLE_CLASS, mxREAL);
        snap = mxGetPr(plhs[1]);
    }

    rc = sssi_rvsTimeSpongeFor2dAw(mxGetPr(prhs[0]), mxGetPr(prhs[1]), (int64_t)nz, (int64_t)nx, (int64_t)nt,
                                   boundary, *mxGetPr(prhs[3]), *mxGetPr(prhs[4]), *mxGetPr(prhs[5]),
                                   mxGetPr(plhs[0]), snap, sssi_mex_mode());
    if (rc != SSSI_OK) mexErrMsgIdAndTxt("sssi:rvsTimeSpongeFor2dAw", "%s", sssi_last_error());
}
