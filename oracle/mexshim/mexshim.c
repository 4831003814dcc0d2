/*
 * Project-written implementation of the MATLAB mx/mex subset declared in
 * mex.h.  TEST INFRASTRUCTURE ONLY: linked into the reference gateways built
 * under oracle/_ref/ and into this project's gateways when tests drive them.
 *
 * Besides the MATLAB API, it exports a small harness (shim_*) that ctypes
 * uses to build mxArrays, call mexFunction with MATLAB's error semantics, and
 * read results back.
 */
#include "mex.h"

#include <math.h>
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define SHIM_MAXDIM 8

struct shim_mxArray {
    mwSize ndim;
    mwSize dims[SHIM_MAXDIM];
    double *data;
    int owns_data; /* 1: data freed by mxDestroyArray */
};

/* ---- mxCalloc bookkeeping: MATLAB frees these when the MEX call returns ---- */
typedef struct shim_block {
    void *p;
    struct shim_block *next;
} shim_block;

static shim_block *g_blocks = NULL;
static jmp_buf g_errjmp;
static int g_in_call = 0;
static char g_errmsg[1024];

static void track(void *p) {
    shim_block *b = (shim_block *)malloc(sizeof(shim_block));
    b->p = p;
    b->next = g_blocks;
    g_blocks = b;
}

static int untrack(void *p) {
    shim_block **pp = &g_blocks;
    while (*pp) {
        if ((*pp)->p == p) {
            shim_block *dead = *pp;
            *pp = dead->next;
            free(dead);
            return 1;
        }
        pp = &(*pp)->next;
    }
    return 0;
}

static void release_all_tracked(void) {
    while (g_blocks) {
        shim_block *b = g_blocks;
        g_blocks = b->next;
        free(b->p);
        free(b);
    }
}

void *mxCalloc(mwSize n, mwSize size) {
    void *p = calloc(n ? n : 1, size ? size : 1);
    if (!p) mexErrMsgTxt("mxCalloc: out of memory");
    track(p);
    return p;
}

void *mxMalloc(mwSize n) {
    void *p = malloc(n ? n : 1);
    if (!p) mexErrMsgTxt("mxMalloc: out of memory");
    track(p);
    return p;
}

void mxFree(void *p) {
    if (!p) return;
    untrack(p);
    free(p);
}

/* ---- arrays ---- */
static mxArray *new_array(mwSize ndim, const mwSize *dims) {
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    mwSize i, numel = 1;
    if (ndim < 2) ndim = 2;
    a->ndim = ndim;
    for (i = 0; i < ndim && i < SHIM_MAXDIM; i++) {
        a->dims[i] = dims ? dims[i] : 0;
        numel *= a->dims[i];
    }
    /* MATLAB drops trailing singleton dimensions beyond the second */
    while (a->ndim > 2 && a->dims[a->ndim - 1] == 1) a->ndim--;
    a->data = numel ? (double *)calloc(numel, sizeof(double)) : NULL;
    if (numel && !a->data) {
        free(a);
        mexErrMsgTxt("mxCreate: out of memory");
    }
    a->owns_data = 1;
    return a;
}

mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity flag) {
    mwSize d[2];
    (void)flag;
    d[0] = m;
    d[1] = n;
    return new_array(2, d);
}

mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls, mxComplexity flag) {
    (void)cls;
    return mxCreateDoubleMatrix(m, n, flag);
}

mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls, mxComplexity flag) {
    (void)cls;
    (void)flag;
    return new_array(ndim, dims);
}

mxArray *mxCreateDoubleScalar(double value) {
    mxArray *a = mxCreateDoubleMatrix(1, 1, mxREAL);
    a->data[0] = value;
    return a;
}

void mxDestroyArray(mxArray *a) {
    if (!a) return;
    if (a->owns_data && a->data) {
        untrack(a->data);
        free(a->data);
    }
    free(a);
}

double *mxGetPr(const mxArray *a) { return a ? a->data : NULL; }
void *mxGetData(const mxArray *a) { return a ? (void *)a->data : NULL; }

void mxSetData(mxArray *a, void *data) {
    if (a->owns_data && a->data && a->data != data) {
        untrack(a->data);
        free(a->data);
    }
    /* memory handed to an array belongs to the array from now on */
    untrack(data);
    a->data = (double *)data;
    a->owns_data = 1;
}

mwSize mxGetM(const mxArray *a) { return a->dims[0]; }

mwSize mxGetN(const mxArray *a) {
    mwSize i, n = 1;
    for (i = 1; i < a->ndim; i++) n *= a->dims[i];
    return n;
}

void mxSetM(mxArray *a, mwSize m) { a->dims[0] = m; }

void mxSetN(mxArray *a, mwSize n) {
    a->ndim = 2;
    a->dims[1] = n;
}

mwSize mxGetNumberOfDimensions(const mxArray *a) { return a->ndim; }
const mwSize *mxGetDimensions(const mxArray *a) { return a->dims; }

mwSize mxGetNumberOfElements(const mxArray *a) {
    mwSize i, n = 1;
    for (i = 0; i < a->ndim; i++) n *= a->dims[i];
    return n;
}

int mxIsDouble(const mxArray *a) { return a != NULL; }
int mxIsComplex(const mxArray *a) {
    (void)a;
    return 0;
}
double mxGetScalar(const mxArray *a) { return (a && a->data) ? a->data[0] : 0.0; }

/* ---- errors ---- */
void mexErrMsgTxt(const char *msg) {
    snprintf(g_errmsg, sizeof(g_errmsg), "%s", msg ? msg : "");
    if (g_in_call) longjmp(g_errjmp, 1);
    fprintf(stderr, "mexErrMsgTxt outside a gateway call: %s\n", g_errmsg);
    abort();
}

void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...) {
    char buf[900];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    snprintf(g_errmsg, sizeof(g_errmsg), "%s: %s", id ? id : "", buf);
    if (g_in_call) longjmp(g_errjmp, 1);
    fprintf(stderr, "mexErrMsgIdAndTxt outside a gateway call: %s\n", g_errmsg);
    abort();
}

void mexWarnMsgTxt(const char *msg) { fprintf(stderr, "Warning: %s\n", msg); }

int mexPrintf(const char *fmt, ...) {
    int r;
    va_list ap;
    va_start(ap, fmt);
    r = vprintf(fmt, ap);
    va_end(ap);
    return r;
}

/*
 * x = A \ b for square A (column-major n x n) by LU with partial pivoting:
 * unblocked right-looking factorisation with the pivot column scaled by the
 * reciprocal of the pivot (LAPACK dgetf2), then the row interchanges applied to
 * b, a unit-lower forward substitution and an upper back substitution, both
 * column-oriented (LAPACK dgetrs -> dtrsm).
 */
static void shim_lu_solve(int n, const double *Ain, const double *bin, double *x) {
    double *A = (double *)malloc(sizeof(double) * (size_t)n * n);
    int *ipiv = (int *)malloc(sizeof(int) * (size_t)n);
    int i, j, k;
    memcpy(A, Ain, sizeof(double) * (size_t)n * n);
    for (i = 0; i < n; i++) x[i] = bin[i];

    for (k = 0; k < n; k++) {
        int p = k;
        double amax = fabs(A[k + (size_t)k * n]);
        for (i = k + 1; i < n; i++) {
            double a = fabs(A[i + (size_t)k * n]);
            if (a > amax) {
                amax = a;
                p = i;
            }
        }
        ipiv[k] = p;
        if (p != k) {
            for (j = 0; j < n; j++) {
                double t = A[k + (size_t)j * n];
                A[k + (size_t)j * n] = A[p + (size_t)j * n];
                A[p + (size_t)j * n] = t;
            }
        }
        if (A[k + (size_t)k * n] != 0.0) {
            double r = 1.0 / A[k + (size_t)k * n];
            for (i = k + 1; i < n; i++) A[i + (size_t)k * n] *= r;
        }
        for (j = k + 1; j < n; j++) {
            double t = -A[k + (size_t)j * n];
            for (i = k + 1; i < n; i++) A[i + (size_t)j * n] += A[i + (size_t)k * n] * t;
        }
    }
    for (k = 0; k < n; k++) {
        if (ipiv[k] != k) {
            double t = x[k];
            x[k] = x[ipiv[k]];
            x[ipiv[k]] = t;
        }
    }
    for (k = 0; k < n; k++) {
        if (x[k] != 0.0)
            for (i = k + 1; i < n; i++) x[i] -= x[k] * A[i + (size_t)k * n];
    }
    for (k = n - 1; k >= 0; k--) {
        if (x[k] != 0.0) {
            x[k] /= A[k + (size_t)k * n];
            for (i = 0; i < k; i++) x[i] -= x[k] * A[i + (size_t)k * n];
        }
    }
    free(A);
    free(ipiv);
}

int mexCallMATLAB(int nlhs, mxArray *plhs[], int nrhs, mxArray *prhs[], const char *name) {
    if (strcmp(name, "mldivide") != 0) mexErrMsgTxt("mexCallMATLAB: only mldivide is available in this shim");
    if (nrhs != 2 || nlhs < 1) mexErrMsgTxt("mexCallMATLAB(mldivide): needs 2 inputs and 1 output");
    {
        int n = (int)mxGetM(prhs[0]);
        if ((int)mxGetN(prhs[0]) != n || (int)mxGetM(prhs[1]) != n || mxGetN(prhs[1]) != 1)
            mexErrMsgTxt("mexCallMATLAB(mldivide): square system with one right-hand side only");
        plhs[0] = mxCreateDoubleMatrix((mwSize)n, 1, mxREAL);
        shim_lu_solve(n, prhs[0]->data, prhs[1]->data, plhs[0]->data);
    }
    return 0;
}

/* ---- harness used from Python through ctypes ---- */

/* A new zero-filled double array that owns its data. */
mxArray *shim_array_new(int ndim, const long long *dims) {
    mwSize d[SHIM_MAXDIM];
    int i;
    if (ndim > SHIM_MAXDIM) return NULL;
    for (i = 0; i < ndim; i++) d[i] = (mwSize)dims[i];
    return new_array((mwSize)ndim, d);
}

/* An array over caller memory (not freed by the shim). */
mxArray *shim_array_borrow(int ndim, const long long *dims, double *data) {
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    int i;
    a->ndim = (mwSize)(ndim < 2 ? 2 : ndim);
    for (i = 0; i < ndim && i < SHIM_MAXDIM; i++) a->dims[i] = (mwSize)dims[i];
    if (ndim < 2) a->dims[1] = 1;
    a->data = data;
    a->owns_data = 0;
    return a;
}

void shim_array_free(mxArray *a) { mxDestroyArray(a); }
double *shim_array_data(mxArray *a) { return a ? a->data : NULL; }
int shim_array_ndim(mxArray *a) { return a ? (int)a->ndim : 0; }
long long shim_array_dim(mxArray *a, int k) { return (a && k < (int)a->ndim) ? (long long)a->dims[k] : 1; }
const char *shim_last_error(void) { return g_errmsg; }

/*
 * Calls the gateway linked into this library.  Returns 0, or 1 when the
 * gateway raised a MATLAB error (message from shim_last_error()).  All
 * mxCalloc memory still outstanding is released afterwards, as MATLAB does.
 */
int shim_call(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs) {
    int rc = 0;
    g_errmsg[0] = 0;
    g_in_call = 1;
    if (setjmp(g_errjmp) == 0) {
        mexFunction(nlhs, plhs, nrhs, prhs);
    } else {
        rc = 1;
    }
    g_in_call = 0;
    release_all_tracked();
    return rc;
}

/* dCoef-style coefficients through the same LU the shim uses for mldivide. */
void shim_mldivide(int n, const double *A, const double *b, double *x) { shim_lu_solve(n, A, b, x); }
