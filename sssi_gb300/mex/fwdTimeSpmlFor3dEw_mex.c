/*
 * fwdTimeSpmlFor3dEw_mex.c -- MEX gateway of 3D elastic forward modelling with
 * the simplified PML on the GPU.  The reference computes this in MATLAB only
 * (src/fwdTimeSpmlFor3dEw.m:1-236); with this gateway that file becomes a
 * one-line wrapper:
 *
 *   function [snapshotVzp, snapshotVxp, snapshotVyp, snapshotVzs, snapshotVxs, snapshotVys] = ...
 *       fwdTimeSpmlFor3dEw(vp, vs, source_x, source_y, source_z, nDiffOrder, nBoundary, dz, dx, dy, dt)
 *   [snapshotVzp, snapshotVxp, snapshotVyp, snapshotVzs, snapshotVxs, snapshotVys] = ...
 *       fwdTimeSpmlFor3dEw_mex(vp, vs, source_x, source_y, source_z, nDiffOrder, nBoundary, dz, dx, dy, dt);
 *
 *     vp, vs      nz x nx x ny        P- and S-wave velocities
 *     source_*    nz x nx x ny x nt   dense sources of the three components
 *     snapshots   nz x nx x ny x nt   only the ones the caller asks for (nlhs)
 *
 * The work is done by sssi_fwdTimeSpmlFor3dEw (libsssi_gb300) in fused FP64
 * unless the environment variable SSSI_MEX_MODE is "strict" or "fp32".
 *
 * Build against MATLAB:  mex -I<repo>/include fwdTimeSpmlFor3dEw_mex.c -L<lib> -lsssi_gb300
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
    const mwSize *dims, *d2;
    mwSize nd, nz, nx, ny, nt, snapdims[4];
    int order, boundary, rc, k;
    double *snap[6] = {NULL, NULL, NULL, NULL, NULL, NULL};

    if (nrhs < 11) mexErrMsgTxt("All 11 input arguments shall be provided!");

    dims = mxGetDimensions(prhs[2]);
    nd = mxGetNumberOfDimensions(prhs[2]);
    if (nd < 3) mexErrMsgTxt("The sources must be nz x nx x ny x nt arrays!");
    nz = dims[0];
    nx = dims[1];
    ny = dims[2];
    nt = nd >= 4 ? dims[3] : 1;
    for (k = 3; k <= 4; ++k) {
        d2 = mxGetDimensions(prhs[k]);
        if (mxGetNumberOfDimensions(prhs[k]) != nd || d2[0] != nz || d2[1] != nx || d2[2] != ny ||
            (nd >= 4 && d2[3] != nt))
            mexErrMsgTxt("Size of X-, Y- and Z-direction source must be the same!");
    }
    d2 = mxGetDimensions(prhs[0]);
    if (mxGetNumberOfDimensions(prhs[0]) < 3 || d2[0] != nz || d2[1] != nx || d2[2] != ny)
        mexErrMsgTxt("Dimension of the velocity models and the sources are not the same!");
    order = (int)*mxGetPr(prhs[5]);
    boundary = (int)*mxGetPr(prhs[6]);

    snapdims[0] = nz;
    snapdims[1] = nx;
    snapdims[2] = ny;
    snapdims[3] = nt;
    for (k = 0; k < 6 && k < (nlhs > 0 ? nlhs : 1); ++k) {
        plhs[k] = mxCreateNumericArray(4, snapdims, mxDOUBLE_CLASS, mxREAL);
        snap[k] = mxGetPr(plhs[k]);
    }

    rc = sssi_fwdTimeSpmlFor3dEw(mxGetPr(prhs[0]), mxGetPr(prhs[1]), mxGetPr(prhs[2]), mxGetPr(prhs[3]),
                                 mxGetPr(prhs[4]), (int64_t)nz, (int64_t)nx, (int64_t)ny, (int64_t)nt, order, boundary,
                                 *mxGetPr(prhs[7]), *mxGetPr(prhs[8]), *mxGetPr(prhs[9]), *mxGetPr(prhs[10]), snap[0],
                                 snap[1], snap[2], snap[3], snap[4], snap[5], sssi_mex_mode());
    if (rc != SSSI_OK) mexErrMsgIdAndTxt("sssi:fwdTimeSpmlFor3dEw", "%s", sssi_last_error());
}
