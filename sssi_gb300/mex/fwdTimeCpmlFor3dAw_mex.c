/*
 * fwdTimeCpmlFor3dAw_mex.c -- MEX gateway of 3D acoustic forward modelling on
 * the GPU.  The reference computes this in MATLAB only
 * (src/fwdTimeCpmlFor3dAw.m:1-163); with this gateway that file becomes a
 * one-line wrapper, like src/fd_cmex/fwdTimeCpmlFor2dAw.m:37:
 *
 *   function [data, snapshot] = fwdTimeCpmlFor3dAw(v, source, nDiffOrder, nBoundary, dz, dx, dy, dt)
 *   [data, snapshot] = fwdTimeCpmlFor3dAw_mex(v, source, nDiffOrder, nBoundary, dz, dx, dy, dt);
 *
 *     v        nz x nx x ny        velocity (already padded by extBoundary)
 *     source   nz x nx x ny x nt   dense source
 *     data     nx x ny x nt        top interior face of every step
 *     snapshot nz x nx x ny x nt   interior field of every step (only computed
 *                                  when the caller asks for two outputs)
 *
 * The work is done by sssi_fwdTimeCpmlFor3dAw (libsssi_gb300) in fused FP64
 * unless the environment variable SSSI_MEX_MODE is "fp32".  The MATLAB file
 * always builds the full snapshot; this gateway skips it when nlhs < 2,
 * because at 3D sizes it is the dominant cost (nz*nx*ny*nt doubles).
 *
 * Build against MATLAB:  mex -I<repo>/include fwdTimeCpmlFor3dAw_mex.c -L<lib> -lsssi_gb300
 */
#include <stdlib.h>
#include <string.h>

#include "mex.h"
#include "sssi_gb300.h"

static int sssi_mex_mode(void) {
    const char *m = getenv("SSSI_MEX_MODE");
    if (m && !strcmp(m, "fp32")) return SSSI_MODE_FP32;
    return SSSI_MODE_FP64;
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    const mwSize *dims, *vdims;
    mwSize nd, nz, nx, ny, nt, ddims[3], sdims[4];
    int order, boundary, rc;
    double *snap = NULL;

    if (nrhs < 8) mexErrMsgTxt("All 8 input arguments shall be provided!");

    dims = mxGetDimensions(prhs[1]);
    nd = mxGetNumberOfDimensions(prhs[1]);
    nz = dims[0];
    nx = dims[1];
    ny = nd >= 3 ? dims[2] : 1;
    nt = nd >= 4 ? dims[3] : 1;
    vdims = mxGetDimensions(prhs[0]);
    if (vdims[0] != nz || vdims[1] != nx || (mxGetNumberOfDimensions(prhs[0]) >= 3 ? vdims[2] : 1) != ny)
        mexErrMsgTxt("Velocity model and source grids should have the same z-axis, x-axis and y-axis grids!");
    order = (int)*mxGetPr(prhs[2]);
    boundary = (int)*mxGetPr(prhs[3]);

    ddims[0] = nx;
    ddims[1] = ny;
    ddims[2] = nt;
    plhs[0] = mxCreateNumericArray(3, ddims, mxDOUBLE_CLASS, mxREAL);
    if (nlhs >= 2) {
        sdims[0] = nz;
        sdims[1] = nx;
        sdims[2] = ny;
        sdims[3] = nt;
        plhs[1] = mxCreateNumericArray(4, sdims, mxDOUBLE_CLASS, mxREAL);
        snap = mxGetPr(plhs[1]);
    }

    rc = sssi_fwdTimeCpmlFor3dAw(mxGetPr(prhs[0]), mxGetPr(prhs[1]), (int64_t)nz, (int64_t)nx, (int64_t)ny,
                                 (int64_t)nt, order, boundary, *mxGetPr(prhs[4]), *mxGetPr(prhs[5]),
                                 *mxGetPr(prhs[6]), *mxGetPr(prhs[7]), mxGetPr(plhs[0]), snap, sssi_mex_mode());
    if (rc != SSSI_OK) mexErrMsgIdAndTxt("sssi:fwdTimeCpmlFor3dAw", "%s", sssi_last_error());
}
