// mex.h — a minimal stand-in for MATLAB's MEX API, enough to compile and run
// psd_projection_gb300/matlab/psd_projection_MATLAB.cpp without MATLAB
// (tests/test_mex_source.py).  Only the calls that file makes exist; errors
// raised through mexErrMsgTxt become C++ exceptions carrying the message.
#pragma once
#include <cstddef>

struct mxArray;
enum mxComplexity { mxREAL = 0, mxCOMPLEX = 1 };

size_t mxGetM(const mxArray* a);
size_t mxGetN(const mxArray* a);
double* mxGetPr(const mxArray* a);
bool mxIsDouble(const mxArray* a);
bool mxIsComplex(const mxArray* a);
bool mxIsSparse(const mxArray* a);
bool mxIsChar(const mxArray* a);
char* mxArrayToString(const mxArray* a);
void mxFree(void* p);
mxArray* mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity c);
[[noreturn]] void mexErrMsgTxt(const char* msg);

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);
