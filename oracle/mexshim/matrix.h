/* Test-infrastructure stand-in for MATLAB's matrix.h: everything lives in mex.h. */
#ifndef SSSI_MEXSHIM_MATRIX_H
#define SSSI_MEXSHIM_MATRIX_H
#include "mex.h"
#endif
