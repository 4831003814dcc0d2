/*
 * Minimal stand-in for MATLAB's mex.h / matrix.h, written for this project.
 *
 * TEST INFRASTRUCTURE ONLY.  It lets two kinds of MEX gateway compile and run
 * without MATLAB:
 *   - the reference gateways (src/fd_cmex/*_mex.c), compiled unmodified from
 *     the reference tree into oracle/_ref/ to pin the oracle;
 *   - this project's own gateways (sssi_gb300/mex/*_mex.c), so the drop-in
 *     boundary can be exercised with the same mxArray calling convention.
 *
 * Only the subset of the mx/mex API that those gateways touch is provided.
 * mxArray holds real double data only (mxDOUBLE_CLASS, mxREAL).  Memory from
 * mxCalloc is tracked and released when the gateway call returns, the way
 * MATLAB releases it.  mexErrMsgTxt unwinds to the harness with longjmp,
 * which is how MATLAB's own error exit behaves for the caller.
 * mexCallMATLAB supports "mldivide" on square real systems only, solved by LU
 * with partial pivoting (the algorithm of LAPACK dgetf2 + dgetrs, which is
 * what MATLAB's mldivide uses for a small dense square system).
 */
#ifndef SSSI_MEXSHIM_MEX_H
#define SSSI_MEXSHIM_MEX_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef size_t mwSize;
typedef size_t mwIndex;

typedef enum { mxUNKNOWN_CLASS = 0, mxDOUBLE_CLASS = 6 } mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

typedef struct shim_mxArray mxArray;

/* array creation / destruction */
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity flag);
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls, mxComplexity flag);
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls, mxComplexity flag);
mxArray *mxCreateDoubleScalar(double value);
void mxDestroyArray(mxArray *a);

/* accessors */
double *mxGetPr(const mxArray *a);
void *mxGetData(const mxArray *a);
void mxSetData(mxArray *a, void *data);
mwSize mxGetM(const mxArray *a);
mwSize mxGetN(const mxArray *a);
void mxSetM(mxArray *a, mwSize m);
void mxSetN(mxArray *a, mwSize n);
mwSize mxGetNumberOfDimensions(const mxArray *a);
const mwSize *mxGetDimensions(const mxArray *a);
mwSize mxGetNumberOfElements(const mxArray *a);
int mxIsDouble(const mxArray *a);
int mxIsComplex(const mxArray *a);
double mxGetScalar(const mxArray *a);

/* memory */
void *mxCalloc(mwSize n, mwSize size);
void *mxMalloc(mwSize n);
void mxFree(void *p);

/* errors and callbacks */
void mexErrMsgTxt(const char *msg);
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
void mexWarnMsgTxt(const char *msg);
int mexPrintf(const char *fmt, ...);
int mexCallMATLAB(int nlhs, mxArray *plhs[], int nrhs, mxArray *prhs[], const char *name);

#define mxAssert(expr, msg) ((void)0)
#define mxAssertS(expr, msg) ((void)0)

/* the gateway every MEX file defines */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);

#ifdef __cplusplus
}
#endif

#endif /* SSSI_MEXSHIM_MEX_H */
