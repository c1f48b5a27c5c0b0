// dropin_caller.cpp — a program written against the reference library's C++
// headers (include/psd_projection/*.h), the way its gtest suite calls them
// (test/composite_FP32_test.hpp:201-247, test/lanczos_test.hpp:8-42): its own
// cuBLAS and cuSOLVER handles, a non-default stream set on both, device
// matrices it allocates itself.  tests/test_gpu_dropin.py compiles it against
// libpsdgb.so, runs it and checks what it writes.
//
// Usage: dropin_caller DIR.  Reads DIR/x300.bin (300 x 300), DIR/x1000.bin,
// DIR/x1024.bin and DIR/kat5.bin (FP64, column-major); writes DIR/<name>.bin
// results and prints one "key value..." line per check.
#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <cstdio>
#include <string>
#include <vector>

#include "psd_projection/composite_FP16.h"
#include "psd_projection/composite_FP32.h"
#include "psd_projection/composite_FP32_emulated.h"
#include "psd_projection/eig_FP32_psd.h"
#include "psd_projection/eig_FP64_psd.h"
#include "psd_projection/lanczos.h"
#include "psdgb.h"

namespace {

std::string g_dir;

std::vector<double> load(const char* name, size_t count) {
    std::vector<double> v(count);
    FILE* f = std::fopen((g_dir + "/" + name).c_str(), "rb");
    if (!f || std::fread(v.data(), sizeof(double), count, f) != count) {
        std::fprintf(stderr, "cannot read %s\n", name);
        std::exit(2);
    }
    std::fclose(f);
    return v;
}

void save(const char* name, const std::vector<double>& v) {
    FILE* f = std::fopen((g_dir + "/" + name).c_str(), "wb");
    if (!f || std::fwrite(v.data(), sizeof(double), v.size(), f) != v.size()) {
        std::fprintf(stderr, "cannot write %s\n", name);
        std::exit(2);
    }
    std::fclose(f);
}

#define CK(x)                                                                          \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess) {                                                       \
            std::fprintf(stderr, "%s failed: %s\n", #x, cudaGetErrorString(e_));       \
            std::exit(3);                                                              \
        }                                                                              \
    } while (0)

size_t free_bytes() {
    size_t fr = 0, tot = 0;
    CK(cudaMemGetInfo(&fr, &tot));
    return fr;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    g_dir = argv[1];
    cublasHandle_t blas = nullptr;
    cusolverDnHandle_t solver = nullptr;
    if (cublasCreate(&blas) != CUBLAS_STATUS_SUCCESS || cusolverDnCreate(&solver) != CUSOLVER_STATUS_SUCCESS) return 4;
    cudaStream_t stream = nullptr;
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    cublasSetStream(blas, stream);
    cusolverDnSetStream(solver, stream);

    // The three auto-scaled composite methods on a 300 x 300 matrix.
    {
        const int n = 300;
        const std::vector<double> x = load("x300.bin", size_t(n) * n);
        double* d = nullptr;
        CK(cudaMalloc(&d, sizeof(double) * n * n));
        std::vector<double> out(size_t(n) * n);
        struct {
            const char* name;
            void (*fn)(cublasHandle_t, cusolverDnHandle_t, double*, int);
        } methods[] = {
            {"composite_FP32_auto_scale",
             [](cublasHandle_t h, cusolverDnHandle_t s, double* m, int k) { composite_FP32_auto_scale(h, s, m, k); }},
            {"composite_FP16_auto_scale",
             [](cublasHandle_t h, cusolverDnHandle_t s, double* m, int k) { composite_FP16_auto_scale(h, s, m, k); }},
            {"composite_FP32_emulated_auto_scale",
             [](cublasHandle_t h, cusolverDnHandle_t s, double* m, int k) {
                 composite_FP32_emulated_auto_scale(h, s, m, k);
             }},
        };
        for (auto& m : methods) {
            CK(cudaMemcpy(d, x.data(), sizeof(double) * n * n, cudaMemcpyHostToDevice));
            m.fn(blas, solver, d, n);
            // The call has finished: the result is read with a plain copy.
            CK(cudaMemcpy(out.data(), d, sizeof(double) * n * n, cudaMemcpyDeviceToHost));
            save((std::string(m.name) + ".bin").c_str(), out);
            std::printf("ran %s\n", m.name);
        }

        // eig_FP64_psd / eig_FP32_psd with the eigenvalues returned in a
        // device array the caller frees.
        for (int fp64 = 1; fp64 >= 0; --fp64) {
            CK(cudaMemcpy(d, x.data(), sizeof(double) * n * n, cudaMemcpyHostToDevice));
            double* eigs = fp64 ? eig_FP64_psd(solver, blas, d, n, true) : eig_FP32_psd(solver, blas, d, n, true);
            if (!eigs) {
                std::printf("eig_returned_null %d\n", fp64);
                continue;
            }
            std::vector<double> w(n);
            CK(cudaMemcpy(w.data(), eigs, sizeof(double) * n, cudaMemcpyDeviceToHost));
            CK(cudaFree(eigs));
            CK(cudaMemcpy(out.data(), d, sizeof(double) * n * n, cudaMemcpyDeviceToHost));
            save(fp64 ? "eig_FP64_psd.bin" : "eig_FP32_psd.bin", out);
            save(fp64 ? "eig_FP64_values.bin" : "eig_FP32_values.bin", w);
        }
        // Without eigenvalues the call returns no array.
        CK(cudaMemcpy(d, x.data(), sizeof(double) * n * n, cudaMemcpyHostToDevice));
        std::printf("eig_without_values_null %d\n", eig_FP64_psd(solver, blas, d, n) == nullptr ? 1 : 0);
        CK(cudaFree(d));
    }

    // approximate_two_norm on the reference's 5 x 5 known-answer matrix.
    {
        const std::vector<double> a = load("kat5.bin", 25);
        double* d = nullptr;
        CK(cudaMalloc(&d, sizeof(double) * 25));
        CK(cudaMemcpy(d, a.data(), sizeof(double) * 25, cudaMemcpyHostToDevice));
        double lo = 0.0, up = 0.0;
        approximate_two_norm(blas, solver, d, 5, &lo, &up, 50, 1e-6);
        std::printf("lanczos %.17g %.17g\n", lo, up);
        CK(cudaFree(d));
    }

    // composite_FP32 with a caller workspace of exactly 3 n^2 floats, the size
    // the reference documents.  n = 1024 (a multiple of 128): the library's
    // layout fits and the call allocates nothing.  n = 1000: it does not fit
    // (the operands are padded to 1024), and the library takes its own cached
    // workspace instead.
    for (int n : {1024, 1000}) {
        const std::vector<double> x = load(n == 1024 ? "x1024.bin" : "x1000.bin", size_t(n) * n);
        double* d = nullptr;
        float* ws = nullptr;
        CK(cudaMalloc(&d, sizeof(double) * n * n));
        CK(cudaMalloc(&ws, sizeof(float) * 3 * size_t(n) * n));
        // Warm-up without a workspace (loads the kernels, fills the cache), then drop the cache.
        CK(cudaMemcpy(d, x.data(), sizeof(double) * n * n, cudaMemcpyHostToDevice));
        composite_FP32(blas, d, n);
        psdgb_release_workspace();
        CK(cudaMemcpy(d, x.data(), sizeof(double) * n * n, cudaMemcpyHostToDevice));
        const size_t before = free_bytes();
        composite_FP32(blas, d, n, ws);
        const size_t after = free_bytes();
        std::printf("workspace_n%d_allocated %lld\n", n, static_cast<long long>(before) - static_cast<long long>(after));
        std::vector<double> out(size_t(n) * n);
        CK(cudaMemcpy(out.data(), d, sizeof(double) * n * n, cudaMemcpyDeviceToHost));
        save(n == 1024 ? "composite_FP32_ws1024.bin" : "composite_FP32_ws1000.bin", out);
        CK(cudaFree(ws));
        CK(cudaFree(d));
    }

    // A failing call prints its error and returns; the program goes on, as
    // with the reference's CHECK_* macros (include/psd_projection/check.h:18-57).
    composite_FP32(blas, nullptr, 16);
    std::printf("continued_after_error 1\n");

    cusolverDnDestroy(solver);
    cublasDestroy(blas);
    CK(cudaStreamDestroy(stream));
    return 0;
}
