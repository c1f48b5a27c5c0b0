// psd_projection_MATLAB.cpp — the MATLAB entry point of the library, on the
// C ABI of libpsdgb.so.  Replaces the reference's MEX wrapper
// (MATLAB/psd_projection_MATLAB.cu:62-188) with the same MATLAB interface:
//
//     X = psd_projection_MATLAB(A, method)
//     [X, lambda] = psd_projection_MATLAB(A, 'eig_FP64' | 'eig_FP32')
//
// A is a real, square, double matrix (symmetric; its upper triangle defines
// it).  method is one of the reference's strings: 'composite_FP16',
// 'composite_FP32', 'composite_FP32_emulated' (Lanczos bound, scaling,
// filter, rescaling), 'eig_FP64', 'eig_FP32' (EVD projection; lambda holds
// the unclipped eigenvalues in ascending order).  Anything else is an error,
// with the reference's message.
//
// The reference copies A to the device, creates cuBLAS / cuSOLVER handles,
// runs the method and copies the result back, allocating and freeing every
// buffer per call.  Here one psdgb_project_host call does the copies and the
// projection; the library keeps its device buffers across calls.
//
// Build (MATLAB present):
//     mex -R2018a -I<repo>/include psd_projection_MATLAB.cpp \
//         -L<repo>/psd_projection_gb300 -lpsdgb
#include <cstring>
#include <string>

#include "mex.h"
#include "psdgb.h"

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
    if (nrhs != 2) mexErrMsgTxt("Wrong number of input arguments. Expected 2 inputs: mat, method.");
    if (nlhs > 2) mexErrMsgTxt("Too many output arguments.");
    const mxArray* A = prhs[0];
    if (!mxIsDouble(A) || mxIsComplex(A) || mxIsSparse(A))
        mexErrMsgTxt("The 'mat' input must be a real, dense double matrix.");
    const size_t n = mxGetM(A);
    if (mxGetN(A) != n) mexErrMsgTxt("The 'mat' input must be square.");
    if (!mxIsChar(prhs[1])) mexErrMsgTxt("The 'method' input must be a string.");
    char* method_c = mxArrayToString(prhs[1]);
    if (!method_c) mexErrMsgTxt("Failed to convert 'method' input to string.");
    const std::string method(method_c);
    mxFree(method_c);
    const bool eig = method == "eig_FP64" || method == "eig_FP32";
    if (!eig && method != "composite_FP16" && method != "composite_FP32" && method != "composite_FP32_emulated")
        mexErrMsgTxt("Unknown method. Supported methods: 'composite_FP16', 'composite_FP32', "
                     "'composite_FP32_emulated', 'eig_FP64', and 'eig_FP32'.");

    plhs[0] = mxCreateDoubleMatrix(n, n, mxREAL);
    double* eigs = nullptr;
    if (eig && nlhs > 1) {
        plhs[1] = mxCreateDoubleMatrix(n, 1, mxREAL);
        eigs = mxGetPr(plhs[1]);
    }
    // MATLAB stores A column-major with leading dimension n: the library's layout.
    const psdgb_status st =
        psdgb_project_host(method.c_str(), mxGetPr(A), mxGetPr(plhs[0]), static_cast<int64_t>(n), eigs, nullptr);
    if (st != PSDGB_OK) mexErrMsgTxt(psdgb_last_error());
}
