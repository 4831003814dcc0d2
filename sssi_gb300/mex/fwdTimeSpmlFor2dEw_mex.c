/*
 * fwdTimeSpmlFor2dEw_mex.c -- MEX gateway of 2D elastic forward modelling with
 * the simplified PML on the GPU.  The reference computes this in MATLAB only
 * (src/fwdTimeSpmlFor2dEw.m:1-103); with this gateway that file becomes a
 * one-line wrapper:
 *
 *   function [snapshotVzp, snapshotVxp, snapshotVzs, snapshotVxs] = ...
 *       fwdTimeSpmlFor2dEw(vp, vs, source, nDiffOrder, nBoundary, dz, dx, dt)
 *   [snapshotVzp, snapshotVxp, snapshotVzs, snapshotVxs] = ...
 *       fwdTimeSpmlFor2dEw_mex(vp, vs, source, nDiffOrder, nBoundary, dz, dx, dt);
 *
 *     vp, vs     nz x nx         P- and S-wave velocities
 *     source     nz x nx x nt    dense source (added to both P components)
 *     snapshots  nz x nx x nt    only the ones the caller asks for (nlhs)
 *
 * The work is done by sssi_fwdTimeSpmlFor2dEw (libsssi_gb300) in fused FP64
 * unless the environment variable SSSI_MEX_MODE is "strict" (the MATLAB file's
 * and diffOperator_mex's rounding sequence) or "fp32".
 *
 * Build against MATLAB:  mex -I<repo>/include fwdTimeSpmlFor2dEw_mex.c -L<lib> -lsssi_gb300
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
    int order, boundary, rc, k;
    double *snap[4] = {NULL, NULL, NULL, NULL};

    if (nrhs < 8) mexErrMsgTxt("All 8 input arguments shall be provided!");

    dims = mxGetDimensions(prhs[2]);
    nd = mxGetNumberOfDimensions(prhs[2]);
    nz = dims[0];
    nx = dims[1];
    nt = nd >= 3 ? dims[2] : 1;
    if (mxGetM(prhs[0]) != nz || mxGetN(prhs[0]) != nx || mxGetM(prhs[1]) != nz || mxGetN(prhs[1]) != nx)
        mexErrMsgTxt("Dimension of P-wave and S-wave velocity models and the source are not the same!");
    order = (int)*mxGetPr(prhs[3]);
    boundary = (int)*mxGetPr(prhs[4]);

    snapdims[0] = nz;
    snapdims[1] = nx;
    snapdims[2] = nt;
    for (k = 0; k < 4 && k < (nlhs > 0 ? nlhs : 1); ++k) {
        plhs[k] = mxCreateNumericArray(3, snapdims, mxDOUBLE_CLASS, mxREAL);
        snap[k] = mxGetPr(plhs[k]);
    }

    rc = sssi_fwdTimeSpmlFor2dEw(mxGetPr(prhs[0]), mxGetPr(prhs[1]), mxGetPr(prhs[2]), (int64_t)nz, (int64_t)nx,
                                 (int64_t)nt, order, boundary, *mxGetPr(prhs[5]), *mxGetPr(prhs[6]),
                                 *mxGetPr(prhs[7]), snap[0], snap[1], snap[2], snap[3], sssi_mex_mode());
    if (rc != SSSI_OK) mexErrMsgIdAndTxt("sssi:fwdTimeSpmlFor2dEw", "%s", sssi_last_error());
}
