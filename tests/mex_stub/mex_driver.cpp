// mex_driver.cpp — runs the MEX entry point the way MATLAB would call it, on
// arrays of this stand-in runtime (tests/mex_stub/mex.h).
// Usage: mex_driver IN.bin N METHOD OUT.bin [EIGS.bin]
//   IN.bin: N x N doubles, column-major.  Prints "error: <message>" and
//   exits 3 when the entry point raises an error.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "mex.h"

struct mxArray {
    size_t m = 0, n = 0;
    std::vector<double> data;
    bool is_char = false;
    std::string str;
};

size_t mxGetM(const mxArray* a) { return a->m; }
size_t mxGetN(const mxArray* a) { return a->n; }
double* mxGetPr(const mxArray* a) { return const_cast<double*>(a->data.data()); }
bool mxIsDouble(const mxArray* a) { return !a->is_char; }
bool mxIsComplex(const mxArray*) { return false; }
bool mxIsSparse(const mxArray*) { return false; }
bool mxIsChar(const mxArray* a) { return a->is_char; }
char* mxArrayToString(const mxArray* a) {
    if (!a->is_char) return nullptr;
    char* s = static_cast<char*>(std::malloc(a->str.size() + 1));
    std::memcpy(s, a->str.c_str(), a->str.size() + 1);
    return s;
}
void mxFree(void* p) { std::free(p); }
mxArray* mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity) {
    auto* a = new mxArray();
    a->m = m;
    a->n = n;
    a->data.assign(m * n, 0.0);
    return a;
}
void mexErrMsgTxt(const char* msg) { throw std::runtime_error(msg); }

int main(int argc, char** argv) {
    if (argc < 5) return 2;
    const size_t n = std::strtoull(argv[2], nullptr, 10);
    mxArray A;
    A.m = A.n = n;
    A.data.resize(n * n);
    FILE* f = std::fopen(argv[1], "rb");
    if (!f || std::fread(A.data.data(), sizeof(double), n * n, f) != n * n) return 2;
    std::fclose(f);
    mxArray M;
    M.is_char = true;
    M.str = argv[3];
    const mxArray* prhs[2] = {&A, &M};
    mxArray* plhs[2] = {nullptr, nullptr};
    const int nlhs = argc > 5 ? 2 : 1;
    try {
        mexFunction(nlhs, plhs, 2, prhs);
    } catch (const std::exception& e) {
        std::printf("error: %s\n", e.what());
        return 3;
    }
    for (int k = 0; k < nlhs; ++k) {
        if (!plhs[k]) continue;
        FILE* o = std::fopen(argv[4 + k], "wb");
        if (!o) return 2;
        std::fwrite(plhs[k]->data.data(), sizeof(double), plhs[k]->data.size(), o);
        std::fclose(o);
        delete plhs[k];
    }
    std::printf("ok\n");
    return 0;
}
