/*
 * diffOperator_mex.c -- MEX gateway of the staggered first derivative on the
 * GPU.  Drop-in replacement for src/fd_cmex/diffOperator_mex.c:29-213: same
 * symbol, inputs and output, so src/fd_cmex/diffOperator.m and the MATLAB code
 * that calls diffOperator (the elastic and 3D propagators) run unchanged.
 *
 *   diffData = diffOperator_mex(data, c, d, dim)
 *     data   n1 x n2 or n1 x n2 x n3
 *     c      the differentiation coefficients (order = numel(c))
 *     d      distance per sample
 *     dim    dimension (default 1); as in the reference, a 2D array takes any
 *            dim other than 1 as 2, a 3D array any dim other than 1 or 2 as 3
 *     diffData  data's size with dimension dim shortened by 2*order - 1
 *
 * The work is done by sssi_diffOperator (libsssi_gb300), in fused FP64
 * (within 1e-12 relative L2 of the reference) unless the environment variable
 * SSSI_MEX_MODE is "strict" (the reference's rounding: bit-identical).
 */
#include <stdlib.h>
#include <string.h>

#include "mex.h"
#include "sssi_gb300.h"

static int sssi_mex_mode(void) {
    const char *m = getenv("SSSI_MEX_MODE");
    if (m && !strcmp(m, "strict")) return SSSI_MODE_FP64_STRICT;
    return SSSI_MODE_FP64;
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    const mwSize *pdims;
    mwSize ndims, order, outdims[3];
    int64_t dims[3];
    int dim, l, k, rc;
    (void)nlhs;

    if (nrhs < 3) mexErrMsgTxt("Input data, finite difference coefficients and distance per sample should be all provided!");
    dim = nrhs < 4 ? 1 : (int)*mxGetPr(prhs[3]);
    ndims = mxGetNumberOfDimensions(prhs[0]);
    if (ndims > 3) mexErrMsgTxt("diffOperator: data must be a 2D or 3D array!");
    order = mxGetNumberOfElements(prhs[1]);
    if (order < 1) mexErrMsgTxt("diffOperator: at least one finite difference coefficient is needed!");
    l = 2 * (int)order - 1;
    pdims = mxGetDimensions(prhs[0]);
    if (ndims <= 2)
        dim = dim == 1 ? 1 : 2;
    else
        dim = (dim == 1 || dim == 2) ? dim : 3;
    for (k = 0; k < 3; ++k) dims[k] = k < (int)ndims ? (int64_t)pdims[k] : 1;
    if (dims[dim - 1] < l) mexErrMsgTxt("diffOperator: the stencil is longer than the dimension!");
    for (k = 0; k < 3; ++k) outdims[k] = (mwSize)dims[k];
    outdims[dim - 1] -= (mwSize)l;
    if (ndims <= 2)
        plhs[0] = mxCreateDoubleMatrix(outdims[0], outdims[1], mxREAL);
    else
        plhs[0] = mxCreateNumericArray(3, outdims, mxDOUBLE_CLASS, mxREAL);
    rc = sssi_diffOperator(mxGetPr(prhs[0]), ndims <= 2 ? 2 : 3, dims, mxGetPr(prhs[1]), (int)order,
                           *mxGetPr(prhs[2]), dim, mxGetPr(plhs[0]), sssi_mex_mode());
    if (rc != SSSI_OK) mexErrMsgIdAndTxt("sssi:diffOperator", "%s", sssi_last_error());
}
