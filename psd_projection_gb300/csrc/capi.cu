// capi.cu — the extern "C" entry points of libpsdgb.so (declared in include/psdgb.h).
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "internal.h"

namespace psdgb {

psdgb_status composite_run(DeviceState* ds, int precision, int schedule, double* mat, int64_t n, void* ws,
                           bool auto_scale, int64_t max_iter, double tol, uint64_t seed, int residual_mode,
                           void* lz_state, cudaStream_t s, double* up_out);
psdgb_status eigenpairs_run(DeviceState* ds, cublasHandle_t blas, cusolverDnHandle_t solver, const double* A,
                            int64_t n, int64_t k, bool upper_only, int64_t max_iter, double ortho_tol, uint64_t seed,
                            int64_t* r_out, double* d_vals, double* d_vecs, double* upper_out, cudaStream_t s);
psdgb_status lobpcg_run(DeviceState* ds, cublasHandle_t blas, cusolverDnHandle_t solver, const double* A, double* V,
                        double* D, int64_t n, int64_t m, bool warmstart, int maxiter, double tol, uint64_t seed,
                        int* iters_out, cudaStream_t s);

namespace {

thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};
std::mutex g_mu;                         // guards g_states and the cached workspaces
std::map<int, DeviceState*> g_states;   // one per device, kept until exit
std::recursive_mutex g_call_mu;          // one library call at a time uses the cached workspaces

constexpr uint64_t kDefaultSeed = 0x5eed5eedull;

// Product timing state (psdgb_product_timing_*).
struct TimingState {
    bool on = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending, spare;
    std::vector<double> pending_flops;
    double ms = 0.0, flops = 0.0;
    uint64_t launches = 0;
    cudaEvent_t cur = nullptr;
};
TimingState g_timing;
std::mutex g_timing_mu;

// Grow-only cached device buffer.
psdgb_status ensure_buffer(void** ptr, size_t* have, size_t need) {
    if (*have >= need && *ptr != nullptr) return PSDGB_OK;
    if (*ptr) {
        cudaDeviceSynchronize();
        cudaFree(*ptr);
        *ptr = nullptr;
        *have = 0;
    }
    if (need == 0) return PSDGB_OK;
    cudaError_t e = cudaMalloc(ptr, need);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        set_error(std::string("workspace allocation of ") + std::to_string(need) + " bytes failed: " +
                  cudaGetErrorString(e));
        return PSDGB_ERR_OUT_OF_MEMORY;
    }
    *have = need;
    return PSDGB_OK;
}

struct Handles {
    cublasHandle_t blas = nullptr;
    cusolverDnHandle_t solver = nullptr;
};
Handles& handles_for_device(int dev) {
    static std::map<int, Handles> hs;
    std::lock_guard<std::mutex> lk(g_mu);
    Handles& h = hs[dev];
    if (!h.blas) cublasCreate(&h.blas);
    if (!h.solver) cusolverDnCreate(&h.solver);
    return h;
}

}  // namespace

thread_local int g_sm_cap = 0;

void set_error(const std::string& msg) { g_last_error = msg; }

psdgb_status cuda_fail(cudaError_t e, const char* what) {
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? PSDGB_ERR_OUT_OF_MEMORY : PSDGB_ERR_CUDA;
}

void count_launch(uint64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

psdgb_status device_state(DeviceState** out) {
    int dev = 0;
    PSDGB_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_states.find(dev);
    if (it != g_states.end()) {
        *out = it->second;
        return PSDGB_OK;
    }
    DeviceState* ds = new DeviceState();
    ds->device = dev;
    cudaDeviceProp prop;
    PSDGB_CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
    ds->sm_count = prop.multiProcessorCount;
    ds->cc_major = prop.major;
    ds->cc_minor = prop.minor;
    PSDGB_CUDA_TRY(cudaMalloc(&ds->d_error, 256));
    PSDGB_CUDA_TRY(cudaMemset(ds->d_error, 0, 256));
    g_states[dev] = ds;
    *out = ds;
    return PSDGB_OK;
}

void product_timing_begin(cudaStream_t s) {
    std::lock_guard<std::mutex> lk(g_timing_mu);
    if (!g_timing.on) return;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!g_timing.spare.empty()) {
        e0 = g_timing.spare.back().first;
        e1 = g_timing.spare.back().second;
        g_timing.spare.pop_back();
    } else {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
    }
    cudaEventRecord(e0, s);
    g_timing.pending.push_back({e0, e1});
    g_timing.pending_flops.push_back(0.0);
}

void product_timing_end(cudaStream_t s, double mma_flops) {
    std::lock_guard<std::mutex> lk(g_timing_mu);
    if (!g_timing.on || g_timing.pending.empty()) return;
    cudaEventRecord(g_timing.pending.back().second, s);
    g_timing.pending_flops.back() = mma_flops;
}

void product_timing_collect() {
    std::lock_guard<std::mutex> lk(g_timing_mu);
    for (size_t i = 0; i < g_timing.pending.size(); ++i) {
        float ms = 0.f;
        cudaEventSynchronize(g_timing.pending[i].second);
        if (cudaEventElapsedTime(&ms, g_timing.pending[i].first, g_timing.pending[i].second) == cudaSuccess) {
            g_timing.ms += ms;
            g_timing.flops += g_timing.pending_flops[i];
            g_timing.launches += 1;
        }
        g_timing.spare.push_back(g_timing.pending[i]);
    }
    g_timing.pending.clear();
    g_timing.pending_flops.clear();
}

psdgb_status finish(DeviceState* ds, cudaStream_t stream) {
    PSDGB_CUDA_TRY(cudaStreamSynchronize(stream));
    product_timing_collect();
    int code = 0;
    PSDGB_CUDA_TRY(cudaMemcpy(&code, ds->d_error, sizeof(int), cudaMemcpyDeviceToHost));
    if (code != DEVERR_NONE) {
        PSDGB_CUDA_TRY(cudaMemset(ds->d_error, 0, sizeof(int)));
        set_error("a bounded device-side wait gave up (device error " + std::to_string(code) + ")");
        return PSDGB_ERR_DEVICE_TIMEOUT;
    }
    return PSDGB_OK;
}

}  // namespace psdgb

using namespace psdgb;

namespace {

psdgb_status require_sm103(DeviceState* ds) {
    if (!(ds->cc_major == 10 && ds->cc_minor == 3)) {
        set_error("psdgb kernels are built for sm_103a; device has compute capability " +
                  std::to_string(ds->cc_major) + "." + std::to_string(ds->cc_minor));
        return PSDGB_ERR_UNSUPPORTED;
    }
    return PSDGB_OK;
}

// Caller workspaces feed TMA tensor maps and 16-byte vector accesses.
psdgb_status check_ws_align(const void* p, const char* what) {
    if (p != nullptr && (reinterpret_cast<uintptr_t>(p) & 15u) != 0) {
        set_error(std::string(what) + " must be 16-byte aligned (cudaMalloc gives 256)");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    return PSDGB_OK;
}

// Resolve the composite workspace: the caller's when large enough, else the cache.
psdgb_status resolve_ws(DeviceState* ds, int64_t n, int precision, void* d_ws, size_t ws_bytes, void** out) {
    const size_t need = composite_ws_bytes(n, precision);
    PSDGB_TRY(check_ws_align(d_ws, "the workspace"));
    if (d_ws != nullptr && ws_bytes >= need) {
        *out = d_ws;
        return PSDGB_OK;
    }
    PSDGB_TRY(ensure_buffer(&ds->ws, &ds->ws_bytes, need));
    *out = ds->ws;
    return PSDGB_OK;
}

psdgb_status resolve_lz(DeviceState* ds, int64_t n, int64_t max_iter, void** out) {
    PSDGB_TRY(ensure_buffer(&ds->lz, &ds->lz_bytes, lanczos_state_bytes(n, max_iter)));
    *out = ds->lz;
    return PSDGB_OK;
}

psdgb_status do_eig(DeviceState* ds, int fp64, double* d_mat, int64_t n, double* d_eigs_out, cudaStream_t s) {
    if (n == 0) return PSDGB_OK;
    Handles& h = handles_for_device(ds->device);
    if (cusolverDnSetStream(h.solver, s) != CUSOLVER_STATUS_SUCCESS || cublasSetStream(h.blas, s) != CUBLAS_STATUS_SUCCESS) {
        set_error("cuSOLVER/cuBLAS set stream failed");
        return PSDGB_ERR_SOLVER;
    }
    const int in = static_cast<int>(n);
    const size_t nn = static_cast<size_t>(n) * n;
    // Every call below is checked; the first failure is kept (st, msg) and
    // the later steps are skipped, but the buffers are always freed.
    psdgb_status st = PSDGB_OK;
    std::string msg;
    auto cuda_ok = [&](cudaError_t e, const char* what) {
        if (st == PSDGB_OK && e != cudaSuccess) {
            st = e == cudaErrorMemoryAllocation ? PSDGB_ERR_OUT_OF_MEMORY : PSDGB_ERR_CUDA;
            msg = std::string("eig: ") + what + ": " + cudaGetErrorString(e);
        }
        return st == PSDGB_OK;
    };
    auto lib_ok = [&](bool ok, const char* what) {
        if (st == PSDGB_OK && !ok) {
            st = PSDGB_ERR_SOLVER;
            msg = std::string("eig: ") + what + " failed";
        }
        return st == PSDGB_OK;
    };
    int* d_info = nullptr;
    cuda_ok(cudaMalloc(&d_info, sizeof(int)), "cudaMalloc(info)");
    if (fp64) {
        // src/eig_FP64_psd.cu:24-85: syevd (upper) -> clip -> V diag(max(w,0)) V^T.
        double *V = nullptr, *W = nullptr, *work = nullptr, *VS = nullptr;
        int lwork = 0;
        cuda_ok(cudaMalloc(&V, nn * 8), "cudaMalloc(V)") && cuda_ok(cudaMalloc(&VS, nn * 8), "cudaMalloc(VS)") &&
            cuda_ok(cudaMalloc(&W, n * 8), "cudaMalloc(W)") &&
            cuda_ok(cudaMemcpyAsync(V, d_mat, nn * 8, cudaMemcpyDeviceToDevice, s), "copy of the input") &&
            lib_ok(cusolverDnDsyevd_bufferSize(h.solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, in, V, in,
                                               W, &lwork) == CUSOLVER_STATUS_SUCCESS,
                   "cusolverDnDsyevd_bufferSize") &&
            cuda_ok(cudaMalloc(&work, sizeof(double) * (lwork > 0 ? lwork : 1)), "cudaMalloc(work)") &&
            lib_ok(cusolverDnDsyevd(h.solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, in, V, in, W, work,
                                    lwork, d_info) == CUSOLVER_STATUS_SUCCESS,
                   "cusolverDnDsyevd") &&
            (d_eigs_out == nullptr ||
             cuda_ok(cudaMemcpyAsync(d_eigs_out, W, n * 8, cudaMemcpyDeviceToDevice, s), "copy of the eigenvalues")) &&
            cuda_ok(cudaMemcpyAsync(VS, V, nn * 8, cudaMemcpyDeviceToDevice, s), "copy of the eigenvectors") &&
            cuda_ok(launch_scale_columns_relu(VS, W, n, s), "column scaling");
        const double one = 1.0, zero = 0.0;
        if (st == PSDGB_OK)
            lib_ok(cublasDgemm(h.blas, CUBLAS_OP_N, CUBLAS_OP_T, in, in, in, &one, VS, in, V, in, &zero, d_mat, in) ==
                       CUBLAS_STATUS_SUCCESS,
                   "cublasDgemm");
        cuda_ok(cudaStreamSynchronize(s), "stream synchronisation");
        cudaFree(V); cudaFree(VS); cudaFree(W); cudaFree(work);
    } else {
        // src/eig_FP32_psd.cu:23-96: FP32 copy -> Ssyevd -> clip -> V diag V^T -> FP64.
        float *A = nullptr, *VS = nullptr, *W = nullptr, *work = nullptr, *C = nullptr;
        int lwork = 0;
        cuda_ok(cudaMalloc(&A, nn * 4), "cudaMalloc(A)") && cuda_ok(cudaMalloc(&VS, nn * 4), "cudaMalloc(VS)") &&
            cuda_ok(cudaMalloc(&C, nn * 4), "cudaMalloc(C)") && cuda_ok(cudaMalloc(&W, n * 4), "cudaMalloc(W)") &&
            cuda_ok(launch_f64_to_f32(d_mat, A, static_cast<int64_t>(nn), s), "FP32 copy") &&
            lib_ok(cusolverDnSsyevd_bufferSize(h.solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, in, A, in,
                                               W, &lwork) == CUSOLVER_STATUS_SUCCESS,
                   "cusolverDnSsyevd_bufferSize") &&
            cuda_ok(cudaMalloc(&work, sizeof(float) * (lwork > 0 ? lwork : 1)), "cudaMalloc(work)") &&
            lib_ok(cusolverDnSsyevd(h.solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, in, A, in, W, work,
                                    lwork, d_info) == CUSOLVER_STATUS_SUCCESS,
                   "cusolverDnSsyevd") &&
            (d_eigs_out == nullptr || cuda_ok(launch_f32_to_f64(W, d_eigs_out, n, s), "eigenvalue conversion")) &&
            cuda_ok(cudaMemcpyAsync(VS, A, nn * 4, cudaMemcpyDeviceToDevice, s), "copy of the eigenvectors") &&
            cuda_ok(launch_scale_columns_relu_f32(VS, W, n, s), "column scaling");
        const float one = 1.0f, zero = 0.0f;
        if (st == PSDGB_OK)
            lib_ok(cublasSgemm(h.blas, CUBLAS_OP_N, CUBLAS_OP_T, in, in, in, &one, VS, in, A, in, &zero, C, in) ==
                       CUBLAS_STATUS_SUCCESS,
                   "cublasSgemm") &&
                cuda_ok(launch_f32_to_f64(C, d_mat, static_cast<int64_t>(nn), s), "FP64 conversion");
        cuda_ok(cudaStreamSynchronize(s), "stream synchronisation");
        cudaFree(A); cudaFree(VS); cudaFree(C); cudaFree(W); cudaFree(work);
    }
    if (st == PSDGB_OK) {
        // syevd's info: 0 on success, > 0 when the tridiagonal QR did not converge.
        int info = 0;
        if (cuda_ok(cudaMemcpy(&info, d_info, sizeof(int), cudaMemcpyDeviceToHost), "read of syevd info") &&
            info != 0) {
            st = PSDGB_ERR_SOLVER;
            msg = "syevd reported info = " + std::to_string(info) + (info > 0 ? " (no convergence)" : "");
        }
    }
    cudaFree(d_info);
    if (st != PSDGB_OK) {
        cudaGetLastError();
        set_error(msg);
    }
    return st;
}

bool method_precision(const char* method, int* precision, int* schedule, int* eig64) {
    *eig64 = -1;
    if (!method) return false;
    if (!std::strcmp(method, "composite_FP16")) { *precision = PSDGB_PREC_FP16; *schedule = PSDGB_SCHEDULE_FP16; return true; }
    if (!std::strcmp(method, "composite_FP32")) { *precision = PSDGB_PREC_FP16X3; *schedule = PSDGB_SCHEDULE_FP32; return true; }
    if (!std::strcmp(method, "composite_FP32_emulated")) { *precision = PSDGB_PREC_BF16X9; *schedule = PSDGB_SCHEDULE_FP32; return true; }
    if (!std::strcmp(method, "eig_FP64")) { *eig64 = 1; return true; }
    if (!std::strcmp(method, "eig_FP32")) { *eig64 = 0; return true; }
    return false;
}

}  // namespace

extern "C" {

int psdgb_version(void) { return 10000; }

const char* psdgb_last_error(void) { return g_last_error.c_str(); }

const char* psdgb_precision_name(int precision) {
    switch (precision) {
        case PSDGB_PREC_FP32_SIMT: return "fp32_simt";
        case PSDGB_PREC_FP16: return "fp16";
        case PSDGB_PREC_BF16: return "bf16";
        case PSDGB_PREC_FP16X3: return "fp16x3";
        case PSDGB_PREC_BF16X3: return "bf16x3";
        case PSDGB_PREC_BF16X6: return "bf16x6";
        case PSDGB_PREC_BF16X9: return "bf16x9";
        case PSDGB_PREC_FP8: return "fp8";
        default: return nullptr;
    }
}

size_t psdgb_composite_workspace_size(int64_t n, int precision) { return composite_ws_bytes(n, precision); }

psdgb_status psdgb_release_workspace(void) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    std::lock_guard<std::mutex> lk(g_mu);
    cudaDeviceSynchronize();
    for (auto& kv : g_states) {
        DeviceState* ds = kv.second;
        if (ds->ws) cudaFree(ds->ws);
        if (ds->lz) cudaFree(ds->lz);
        if (ds->stage2) cudaFree(ds->stage2);
        ds->ws = ds->lz = ds->stage2 = nullptr;
        ds->ws_bytes = ds->lz_bytes = ds->stage2_bytes = 0;
    }
    return PSDGB_OK;
}

psdgb_status psdgb_composite(int precision, int schedule, double* d_mat, int64_t n, void* d_ws, size_t ws_bytes,
                             void* stream) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    if (n > 0 && d_mat == nullptr) { set_error("null matrix"); return PSDGB_ERR_INVALID_ARGUMENT; }
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    PSDGB_TRY(require_sm103(ds));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void* ws = nullptr;
    if (n > 0) PSDGB_TRY(resolve_ws(ds, n, precision, d_ws, ws_bytes, &ws));
    PSDGB_TRY(composite_run(ds, precision, schedule, d_mat, n, ws, false, 0, 0.0, 0, 0, nullptr, s, nullptr));
    return finish(ds, s);
}

psdgb_status psdgb_composite_auto_scale(int precision, int schedule, double* d_mat, int64_t n, int64_t max_iter,
                                        double tol, uint64_t seed, int residual_mode, void* d_ws, size_t ws_bytes,
                                        void* stream, double* up_out) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    if (n > 0 && d_mat == nullptr) { set_error("null matrix"); return PSDGB_ERR_INVALID_ARGUMENT; }
    if (max_iter < 0) { set_error("max_iter must be >= 0"); return PSDGB_ERR_INVALID_ARGUMENT; }
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    PSDGB_TRY(require_sm103(ds));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void *ws = nullptr, *lz = nullptr;
    if (n > 0) {
        PSDGB_TRY(resolve_ws(ds, n, precision, d_ws, ws_bytes, &ws));
        PSDGB_TRY(resolve_lz(ds, n, max_iter, &lz));
    }
    PSDGB_TRY(composite_run(ds, precision, schedule, d_mat, n, ws, true, max_iter, tol, seed, residual_mode, lz, s,
                            up_out));
    return finish(ds, s);
}

size_t psdgb_lanczos_state_size(int64_t n, int64_t max_iter) {
    if (n <= 0 || max_iter < 0) return 0;
    return lanczos_state_bytes(n, max_iter);
}

psdgb_status psdgb_composite_auto_scale_async(int precision, int schedule, double* d_mat, int64_t n,
                                              int64_t max_iter, double tol, uint64_t seed, int residual_mode,
                                              const double* d_warm_start, double* d_ritz_out, void* d_ws,
                                              size_t ws_bytes, void* d_lanczos, size_t lanczos_bytes, void* stream) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    if (n < 0 || max_iter < 0) { set_error("n and max_iter must be >= 0"); return PSDGB_ERR_INVALID_ARGUMENT; }
    if (n == 0) return PSDGB_OK;
    if (d_mat == nullptr) { set_error("null matrix"); return PSDGB_ERR_INVALID_ARGUMENT; }
    if (d_ws == nullptr || ws_bytes < composite_ws_bytes(n, precision) || d_lanczos == nullptr ||
        lanczos_bytes < lanczos_state_bytes(n, max_iter)) {
        set_error("psdgb_composite_auto_scale_async needs caller workspaces of at least "
                  "psdgb_composite_workspace_size and psdgb_lanczos_state_size bytes");
        return PSDGB_ERR_WORKSPACE_TOO_SMALL;
    }
    PSDGB_TRY(check_ws_align(d_ws, "the workspace"));
    PSDGB_TRY(check_ws_align(d_lanczos, "the Lanczos state"));
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    PSDGB_TRY(require_sm103(ds));
    return composite_enqueue(ds, precision, schedule, d_mat, n, d_ws, true, max_iter, tol, seed, residual_mode,
                             d_lanczos, static_cast<cudaStream_t>(stream), d_warm_start, d_ritz_out, -1, 0);
}

psdgb_status psdgb_composite_auto_scale_f32(int precision, int schedule, float* d_mat, int64_t n, int64_t max_iter,
                                            double tol, uint64_t seed, int residual_mode, const double* d_warm_start,
                                            double* d_ritz_out, void* d_ws, size_t ws_bytes, void* d_lanczos,
                                            size_t lanczos_bytes, void* stream) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    if (n < 0 || max_iter < 0) { set_error("n and max_iter must be >= 0"); return PSDGB_ERR_INVALID_ARGUMENT; }
    if (n == 0) return PSDGB_OK;
    if (d_mat == nullptr) { set_error("null matrix"); return PSDGB_ERR_INVALID_ARGUMENT; }
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    PSDGB_TRY(require_sm103(ds));
    void* ws = nullptr;
    PSDGB_TRY(resolve_ws(ds, n, precision, d_ws, ws_bytes, &ws));
    PSDGB_TRY(check_ws_align(d_lanczos, "the Lanczos state"));
    void* lz = d_lanczos;
    if (lz == nullptr || lanczos_bytes < lanczos_state_bytes(n, max_iter)) PSDGB_TRY(resolve_lz(ds, n, max_iter, &lz));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PSDGB_TRY(composite_enqueue_f32(ds, precision, schedule, d_mat, n, ws, max_iter, tol, seed, residual_mode, lz, s,
                                    d_warm_start, d_ritz_out));
    // The library's cached buffers are shared with every other call: when this
    // call took them, it finishes before they can be handed out again.
    if (ws == ds->ws || lz == ds->lz) return finish(ds, s);
    return PSDGB_OK;
}

psdgb_status psdgb_composite_mixed_auto_scale(int bulk_precision, int bulk_schedule, int refine_precision,
                                              int refine_steps, double* d_mat, int64_t n, void* stream) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    PrecisionInfo pb{}, pr{};
    // FP8 operands sit beside the FP16 pair (the F16Q8 format), so an FP8 bulk
    // refines with fp16 / fp16x3 products on the same storage.
    const bool fp8_bulk = bulk_precision == PSDGB_PREC_FP8;
    if (!precision_info(bulk_precision, &pb) || !precision_info(refine_precision, &pr) ||
        (fp8_bulk ? pr.fmt != FMT_F16 : pb.fmt != pr.fmt) || refine_steps < 0 || refine_steps > 8) {
        set_error("psdgb_composite_mixed_auto_scale: the bulk and refinement precisions must share an operand "
                  "format (fp16 or fp8 with fp16x3; bf16 with bf16x3/x6/x9) and 0 <= refine_steps <= 8");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (const char* why = schedule_error(bulk_precision, bulk_schedule)) {
        set_error(why);
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (n < 0 || (n > 0 && d_mat == nullptr)) { set_error("bad matrix"); return PSDGB_ERR_INVALID_ARGUMENT; }
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    PSDGB_TRY(require_sm103(ds));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n == 0) return PSDGB_OK;
    void *ws = nullptr, *lz = nullptr;
    PSDGB_TRY(resolve_ws(ds, n, fp8_bulk ? bulk_precision : refine_precision, nullptr, 0, &ws));
    PSDGB_TRY(resolve_lz(ds, n, 20, &lz));
    PSDGB_TRY(composite_enqueue(ds, refine_precision, bulk_schedule, d_mat, n, ws, true, 20, 1e-10, kDefaultSeed,
                                PSDGB_RESIDUAL_REFERENCE, lz, s, nullptr, nullptr, bulk_precision, refine_steps));
    return finish(ds, s);
}

psdgb_status psdgb_selftest_wait_timeout(double limit_seconds, void* stream) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    if (!(limit_seconds >= 0.001 && limit_seconds <= 5.0)) {
        set_error("selftest: limit must be in [0.001, 5] seconds");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PSDGB_CUDA_TRY(launch_wait_selftest(ds->d_error, static_cast<uint64_t>(limit_seconds * 1e9), s));
    return finish(ds, s);
}

psdgb_status psdgb_check_device_error(void) {
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    PSDGB_CUDA_TRY(cudaDeviceSynchronize());
    return finish(ds, nullptr);
}

psdgb_status psdgb_two_norm_ex(const double* d_A, int64_t n, double* lo, double* up, int64_t max_iter, double tol,
                               uint64_t seed, int residual_mode, void* d_ws, size_t ws_bytes, void* stream,
                               double* h_alpha, double* h_beta, int64_t* nb_iter, double* theta) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    if (!lo || !up) { set_error("lo/up must not be null"); return PSDGB_ERR_INVALID_ARGUMENT; }
    if (n < 0 || max_iter < 0) { set_error("n and max_iter must be >= 0"); return PSDGB_ERR_INVALID_ARGUMENT; }
    if (n > 0 && d_A == nullptr) { set_error("null matrix"); return PSDGB_ERR_INVALID_ARGUMENT; }
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    PSDGB_TRY(require_sm103(ds));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    LanczosResult lr;
    if (n > 0) {
        const int64_t ld = (n + 3) / 4 * 4;
        const size_t a32_bytes = sizeof(float) * static_cast<size_t>(n) * ld;
        void* a32 = nullptr;
        PSDGB_TRY(check_ws_align(d_ws, "the workspace"));
        if (d_ws != nullptr && ws_bytes >= a32_bytes) {
            a32 = d_ws;
        } else {
            PSDGB_TRY(ensure_buffer(&ds->ws, &ds->ws_bytes, a32_bytes));
            a32 = ds->ws;
        }
        void* lz = nullptr;
        PSDGB_TRY(resolve_lz(ds, n, max_iter, &lz));
        PSDGB_CUDA_TRY(launch_sym_upper_to_f32(d_A, n, static_cast<float*>(a32), ld, s));
        PSDGB_TRY(lanczos_bound_async(ds, static_cast<float*>(a32), n, ld, max_iter, tol, seed, residual_mode, lz, s,
                                      nullptr, nullptr));
        PSDGB_TRY(lanczos_read(lz, n, max_iter, s, &lr, h_alpha, h_beta));
    } else {
        if (h_alpha) for (int64_t i = 0; i < max_iter; ++i) h_alpha[i] = 0.0;
        if (h_beta) for (int64_t i = 0; i < max_iter; ++i) h_beta[i] = 0.0;
    }
    *lo = lr.lo;
    *up = lr.up;
    if (nb_iter) *nb_iter = lr.nb_iter;
    if (theta) *theta = lr.theta;
    return finish(ds, s);
}

psdgb_status psdgb_two_norm(const double* d_A, int64_t n, double* lo, double* up, int64_t max_iter, double tol,
                            uint64_t seed, int residual_mode, void* d_ws, size_t ws_bytes, void* stream) {
    return psdgb_two_norm_ex(d_A, n, lo, up, max_iter, tol, seed, residual_mode, d_ws, ws_bytes, stream, nullptr,
                             nullptr, nullptr, nullptr);
}

psdgb_status psdgb_eig_psd(int fp64, double* d_mat, int64_t n, double* d_eigs_out, void* stream) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    if (n < 0 || n > 2147483647LL) { set_error("bad matrix size"); return PSDGB_ERR_INVALID_ARGUMENT; }
    if (n > 0 && d_mat == nullptr) { set_error("null matrix"); return PSDGB_ERR_INVALID_ARGUMENT; }
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PSDGB_TRY(do_eig(ds, fp64, d_mat, n, d_eigs_out, s));
    return finish(ds, s);
}

psdgb_status psdgb_project(const char* method, double* d_mat, int64_t n, double* d_eigs_out, void* stream) {
    int precision = 0, schedule = 0, eig64 = -1;
    if (!method_precision(method, &precision, &schedule, &eig64)) {
        set_error("Unknown method. Supported methods: 'composite_FP16', 'composite_FP32', "
                  "'composite_FP32_emulated', 'eig_FP64', and 'eig_FP32'.");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (eig64 >= 0) return psdgb_eig_psd(eig64, d_mat, n, d_eigs_out, stream);
    return psdgb_composite_auto_scale(precision, schedule, d_mat, n, 20, 1e-10, kDefaultSeed, PSDGB_RESIDUAL_REFERENCE,
                                      nullptr, 0, stream, nullptr);
}

psdgb_status psdgb_project_host(const char* method, const double* h_in, double* h_out, int64_t n, double* h_eigs_out,
                                void* stream) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    int precision = 0, schedule = 0, eig64 = -1;
    if (!method_precision(method, &precision, &schedule, &eig64)) {
        set_error("Unknown method. Supported methods: 'composite_FP16', 'composite_FP32', "
                  "'composite_FP32_emulated', 'eig_FP64', and 'eig_FP32'.");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (n < 0) { set_error("bad matrix size"); return PSDGB_ERR_INVALID_ARGUMENT; }
    if (n == 0) return PSDGB_OK;
    if (!h_in || !h_out) { set_error("null host buffer"); return PSDGB_ERR_INVALID_ARGUMENT; }
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t bytes = sizeof(double) * static_cast<size_t>(n) * n;
    // The staging matrix (and the eigenvalue vector) live in a cached buffer
    // after the composite workspace so repeated calls allocate nothing.
    static void* stage = nullptr;
    static size_t stage_bytes = 0;
    const size_t need = bytes + sizeof(double) * static_cast<size_t>(n) + 256;
    PSDGB_TRY(ensure_buffer(&stage, &stage_bytes, need));
    double* d_mat = static_cast<double*>(stage);
    double* d_eigs = reinterpret_cast<double*>(static_cast<char*>(stage) + (bytes + 255) / 256 * 256);
    PSDGB_CUDA_TRY(cudaMemcpyAsync(d_mat, h_in, bytes, cudaMemcpyHostToDevice, s));
    psdgb_status st = psdgb_project(method, d_mat, n, h_eigs_out ? d_eigs : nullptr, stream);
    if (st != PSDGB_OK) return st;
    PSDGB_CUDA_TRY(cudaMemcpyAsync(h_out, d_mat, bytes, cudaMemcpyDeviceToHost, s));
    if (h_eigs_out && eig64 >= 0)
        PSDGB_CUDA_TRY(cudaMemcpyAsync(h_eigs_out, d_eigs, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    PSDGB_CUDA_TRY(cudaStreamSynchronize(s));
    return PSDGB_OK;
}

// A sequence of host matrices through one device: matrix i's host-to-device
// copy, projection and device-to-host copy run on three streams ordered by
// events, with two staging matrices, so the copies of matrices i + 1 and
// i - 1 overlap the projection of matrix i.  Composite methods use the
// asynchronous path (scale kept on the device); EVD methods run one matrix
// after the other.
psdgb_status psdgb_project_host_many(const char* method, const double* const* h_in, double* const* h_out, int64_t n,
                                     int64_t count, void* stream) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    int precision = 0, schedule = 0, eig64 = -1;
    if (!method_precision(method, &precision, &schedule, &eig64)) {
        set_error("Unknown method. Supported methods: 'composite_FP16', 'composite_FP32', "
                  "'composite_FP32_emulated', 'eig_FP64', and 'eig_FP32'.");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (n < 0 || count < 0) { set_error("bad matrix size or count"); return PSDGB_ERR_INVALID_ARGUMENT; }
    if (n == 0 || count == 0) return PSDGB_OK;
    if (!h_in || !h_out) { set_error("null host buffer list"); return PSDGB_ERR_INVALID_ARGUMENT; }
    for (int64_t i = 0; i < count; ++i)
        if (!h_in[i] || !h_out[i]) { set_error("null host buffer"); return PSDGB_ERR_INVALID_ARGUMENT; }
    // The uploads of the next two matrices may run while result i is copied
    // back, so a result may not land in either of their inputs.
    for (int64_t i = 0; i < count; ++i)
        for (int64_t j = i + 1; j <= i + 2 && j < count; ++j)
            if (static_cast<const void*>(h_out[i]) == static_cast<const void*>(h_in[j])) {
                set_error("psdgb_project_host_many: h_out[i] must not be h_in[i + 1] or h_in[i + 2]");
                return PSDGB_ERR_INVALID_ARGUMENT;
            }
    if (eig64 >= 0) {
        for (int64_t i = 0; i < count; ++i) PSDGB_TRY(psdgb_project_host(method, h_in[i], h_out[i], n, nullptr, stream));
        return PSDGB_OK;
    }
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    PSDGB_TRY(require_sm103(ds));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!ds->copy_in) {
        PSDGB_CUDA_TRY(cudaStreamCreateWithFlags(&ds->copy_in, cudaStreamNonBlocking));
        PSDGB_CUDA_TRY(cudaStreamCreateWithFlags(&ds->copy_out, cudaStreamNonBlocking));
        for (int b = 0; b < DeviceState::kHostStages; ++b) {
            PSDGB_CUDA_TRY(cudaEventCreateWithFlags(&ds->in_done[b], cudaEventDisableTiming));
            PSDGB_CUDA_TRY(cudaEventCreateWithFlags(&ds->comp_done[b], cudaEventDisableTiming));
            PSDGB_CUDA_TRY(cudaEventCreateWithFlags(&ds->out_done[b], cudaEventDisableTiming));
        }
    }
    const size_t bytes = sizeof(double) * static_cast<size_t>(n) * n;
    const size_t stride = (bytes + 255) / 256 * 256;
    // Three staging matrices: the upload of step i waits only for the
    // download of step i - 3, so uploads and downloads (two copy streams)
    // both overlap the projections even when a host copy takes most of a
    // projection's time.
    constexpr int S = DeviceState::kHostStages;
    PSDGB_TRY(ensure_buffer(&ds->stage2, &ds->stage2_bytes, S * stride));
    void *ws = nullptr, *lz = nullptr;
    PSDGB_TRY(resolve_ws(ds, n, precision, nullptr, 0, &ws));
    PSDGB_TRY(resolve_lz(ds, n, 20, &lz));
    // Earlier work on the caller's stream (e.g. writes of the host inputs'
    // producers are the caller's business; device-side users of the staging
    // buffers are only these calls) finishes before the first copy.
    PSDGB_CUDA_TRY(cudaEventRecord(ds->comp_done[0], s));
    PSDGB_CUDA_TRY(cudaStreamWaitEvent(ds->copy_in, ds->comp_done[0], 0));
    for (int64_t i = 0; i < count; ++i) {
        const int b = static_cast<int>(i % S);
        double* d = reinterpret_cast<double*>(static_cast<char*>(ds->stage2) + b * stride);
        if (i >= S) PSDGB_CUDA_TRY(cudaStreamWaitEvent(ds->copy_in, ds->out_done[b], 0));
        PSDGB_CUDA_TRY(cudaMemcpyAsync(d, h_in[i], bytes, cudaMemcpyHostToDevice, ds->copy_in));
        PSDGB_CUDA_TRY(cudaEventRecord(ds->in_done[b], ds->copy_in));
        PSDGB_CUDA_TRY(cudaStreamWaitEvent(s, ds->in_done[b], 0));
        PSDGB_TRY(composite_enqueue(ds, precision, schedule, d, n, ws, true, 20, 1e-10, kDefaultSeed,
                                    PSDGB_RESIDUAL_REFERENCE, lz, s, nullptr, nullptr, -1, 0));
        PSDGB_CUDA_TRY(cudaEventRecord(ds->comp_done[b], s));
        PSDGB_CUDA_TRY(cudaStreamWaitEvent(ds->copy_out, ds->comp_done[b], 0));
        PSDGB_CUDA_TRY(cudaMemcpyAsync(h_out[i], d, bytes, cudaMemcpyDeviceToHost, ds->copy_out));
        PSDGB_CUDA_TRY(cudaEventRecord(ds->out_done[b], ds->copy_out));
    }
    PSDGB_CUDA_TRY(cudaStreamWaitEvent(s, ds->out_done[(count - 1) % S], 0));
    return finish(ds, s);
}

psdgb_status psdgb_compute_eigenpairs(const double* d_A, int64_t n, int64_t k, int64_t* r_out, double* d_eigenvalues,
                                      double* d_eigenvectors, int upper_bound_only, int64_t max_iter, double tol,
                                      double ortho_tol, uint64_t seed, double* upper_out, void* stream) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    (void)tol;  // as in the reference, the residual filter compares with ortho_tol (src/lanczos.cu:454)
    if (n <= 0 || d_A == nullptr || k < 0 || max_iter < 0) {
        set_error("compute_eigenpairs: need n > 0, a matrix, k >= 0 and max_iter >= 0");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (!upper_bound_only && k > 0 && (d_eigenvalues == nullptr || d_eigenvectors == nullptr)) {
        set_error("compute_eigenpairs: eigenvalue and eigenvector outputs are required unless upper_bound_only");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    PSDGB_TRY(require_sm103(ds));
    Handles& h = handles_for_device(ds->device);
    return eigenpairs_run(ds, h.blas, h.solver, d_A, n, k, upper_bound_only != 0, max_iter, ortho_tol, seed, r_out,
                          d_eigenvalues, d_eigenvectors, upper_out, static_cast<cudaStream_t>(stream));
}

// src/composite_FP32.cu:193-254 (and the BF16x9 twin, src/composite_FP32_emulated.cu:264-325).
psdgb_status psdgb_composite_auto_scale_deflate(int precision, int schedule, double* d_mat, int64_t n, int64_t k,
                                                double tol, double ortho_tol, uint64_t seed, void* stream) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    PrecisionInfo pi{};
    if (!precision_info(precision, &pi)) {
        set_error("composite_auto_scale_deflate: unknown precision");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (const char* why = schedule_error(precision, schedule)) {
        set_error(why);
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (n < 0 || k < 0 || (n > 0 && d_mat == nullptr)) {
        set_error("composite_auto_scale_deflate: bad matrix or k");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return PSDGB_OK;
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    PSDGB_TRY(require_sm103(ds));
    Handles& h = handles_for_device(ds->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t kk = k < n ? k : n;
    double *vals = nullptr, *vecs = nullptr, *coef = nullptr;
    struct Free {
        double** p[3];
        ~Free() {
            for (double** q : p)
                if (*q) cudaFree(*q);
        }
    } release{{&vals, &vecs, &coef}};
    if (kk > 0 && (cudaMalloc(&vals, sizeof(double) * kk) != cudaSuccess ||
                   cudaMalloc(&vecs, sizeof(double) * kk * n) != cudaSuccess ||
                   cudaMalloc(&coef, sizeof(double) * kk) != cudaSuccess)) {
        cudaGetLastError();
        set_error("composite_auto_scale_deflate: device allocation failed");
        return PSDGB_ERR_OUT_OF_MEMORY;
    }
    // Step 1: the k largest-|lambda| Ritz pairs that pass the reference's filters.
    int64_t r = 0;
    double up_unused = 0.0;
    if (kk > 0)
        PSDGB_TRY(eigenpairs_run(ds, h.blas, h.solver, d_mat, n, kk, false, 0, ortho_tol, seed, &r, vals, vecs,
                                 &up_unused, s));
    (void)tol;
    std::vector<double> hv(static_cast<size_t>(r)), hc(static_cast<size_t>(r));
    if (r > 0) PSDGB_CUDA_TRY(cudaMemcpy(hv.data(), vals, sizeof(double) * r, cudaMemcpyDeviceToHost));
    // Step 2: X -= sum_i lambda_i v_i v_i^T.
    for (int64_t i = 0; i < r; ++i) hc[i] = -hv[i];
    if (r > 0) {
        PSDGB_CUDA_TRY(cudaMemcpyAsync(coef, hc.data(), sizeof(double) * r, cudaMemcpyHostToDevice, s));
        PSDGB_CUDA_TRY(launch_rank_update(d_mat, n, vecs, coef, static_cast<int>(r), s));
    }
    // Step 3: bound of the deflated matrix (100 Lanczos steps), scale 1.1 up + 1e-5.
    double up = 0.0;
    PSDGB_TRY(eigenpairs_run(ds, h.blas, h.solver, d_mat, n, 0, true, 100, 1e-5, seed + 1, nullptr, nullptr, nullptr,
                             &up, s));
    const double scale = up > 0.0 ? 1.1 * up + 1e-5 : 1.0;
    // Step 4: the filter of X / scale, scaled back.
    void* ws = nullptr;
    PSDGB_TRY(resolve_ws(ds, n, precision, nullptr, 0, &ws));
    PSDGB_TRY(composite_enqueue_scaled(ds, precision, schedule, d_mat, n, ws, scale, s));
    // Step 5: add the positive deflated pairs back.
    for (int64_t i = 0; i < r; ++i) hc[i] = hv[i] > 0.0 ? hv[i] : 0.0;
    if (r > 0) {
        PSDGB_CUDA_TRY(cudaMemcpyAsync(coef, hc.data(), sizeof(double) * r, cudaMemcpyHostToDevice, s));
        PSDGB_CUDA_TRY(launch_rank_update(d_mat, n, vecs, coef, static_cast<int>(r), s));
    }
    return finish(ds, s);
}

psdgb_status psdgb_lobpcg(const double* d_A, double* d_V, double* d_D, int64_t n, int64_t m, int warmstart,
                          int maxiter, double tol, uint64_t seed, int* iterations_out, void* stream) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    if (d_A == nullptr || d_V == nullptr || d_D == nullptr || maxiter < 0) {
        set_error("lobpcg: null pointer or negative maxiter");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    Handles& h = handles_for_device(ds->device);
    return lobpcg_run(ds, h.blas, h.solver, d_A, d_V, d_D, n, m, warmstart != 0, maxiter, tol, seed, iterations_out,
                      static_cast<cudaStream_t>(stream));
}

namespace {

// The two-ended deflation of src/eig_FP64_psd.cu:87-177 and
// src/composite_FP16.cu:276-380: the k largest (LOBPCG on X) and k smallest
// (LOBPCG on -X) eigenpairs are subtracted, the rest is projected (`eig`: the
// FP64 EVD projection; else the Lanczos bound, scaling by 1.1 up + 1e-5 and
// the composite filter), and the positive parts of both ends are added back.
psdgb_status deflate_two_ends(bool eig, int precision, int schedule, double* d_mat, int64_t n, int64_t k, int maxiter,
                              double tol, uint64_t seed, cudaStream_t s) {
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    if (!eig) PSDGB_TRY(require_sm103(ds));
    Handles& h = handles_for_device(ds->device);
    double *Vt = nullptr, *Dt = nullptr, *Vb = nullptr, *Db = nullptr, *coef = nullptr;
    struct Free {
        double** p[5];
        ~Free() {
            for (double** q : p)
                if (*q) cudaFree(*q);
        }
    } release{{&Vt, &Dt, &Vb, &Db, &coef}};
    if (cudaMalloc(&Vt, sizeof(double) * n * k) != cudaSuccess || cudaMalloc(&Vb, sizeof(double) * n * k) != cudaSuccess ||
        cudaMalloc(&Dt, sizeof(double) * k) != cudaSuccess || cudaMalloc(&Db, sizeof(double) * k) != cudaSuccess ||
        cudaMalloc(&coef, sizeof(double) * k) != cudaSuccess) {
        cudaGetLastError();
        set_error("deflate: device allocation failed");
        return PSDGB_ERR_OUT_OF_MEMORY;
    }
    const int kk = static_cast<int>(k);
    const int64_t nn = n * n;
    std::vector<double> top(k), bot(k), c(k);
    // Largest: X -= lambda v v^T.
    PSDGB_TRY(lobpcg_run(ds, h.blas, h.solver, d_mat, Vt, Dt, n, k, false, maxiter, tol, seed, nullptr, s));
    PSDGB_CUDA_TRY(cudaMemcpy(top.data(), Dt, sizeof(double) * k, cudaMemcpyDeviceToHost));
    for (int i = 0; i < kk; ++i) c[i] = -top[i];
    PSDGB_CUDA_TRY(cudaMemcpyAsync(coef, c.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    PSDGB_CUDA_TRY(launch_rank_update(d_mat, n, Vt, coef, kk, s));
    // Smallest: LOBPCG on -X gives mu = -lambda; X += mu v v^T.
    PSDGB_CUDA_TRY(launch_scale_inplace(d_mat, nn, -1.0, s));
    PSDGB_TRY(lobpcg_run(ds, h.blas, h.solver, d_mat, Vb, Db, n, k, false, maxiter, tol, seed, nullptr, s));
    PSDGB_CUDA_TRY(launch_scale_inplace(d_mat, nn, -1.0, s));
    PSDGB_CUDA_TRY(cudaMemcpy(bot.data(), Db, sizeof(double) * k, cudaMemcpyDeviceToHost));
    PSDGB_CUDA_TRY(cudaMemcpyAsync(coef, bot.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    PSDGB_CUDA_TRY(launch_rank_update(d_mat, n, Vb, coef, kk, s));
    // The rest.
    if (eig) {
        PSDGB_TRY(do_eig(ds, 1, d_mat, n, nullptr, s));
    } else {
        double lo = 0.0, up = 0.0;
        PSDGB_TRY(psdgb_two_norm(d_mat, n, &lo, &up, 20, 1e-10, seed, PSDGB_RESIDUAL_REFERENCE, nullptr, 0, s));
        const double scale = up > 0.0 ? 1.1 * up + 1e-5 : 1.0;
        void* ws = nullptr;
        PSDGB_TRY(resolve_ws(ds, n, precision, nullptr, 0, &ws));
        PSDGB_TRY(composite_enqueue_scaled(ds, precision, schedule, d_mat, n, ws, scale, s));
    }
    // Add back the positive parts: max(lambda_top, 0) and max(-mu_bottom, 0).
    for (int i = 0; i < kk; ++i) c[i] = top[i] > 0.0 ? top[i] : 0.0;
    PSDGB_CUDA_TRY(cudaMemcpyAsync(coef, c.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    PSDGB_CUDA_TRY(launch_rank_update(d_mat, n, Vt, coef, kk, s));
    PSDGB_CUDA_TRY(cudaStreamSynchronize(s));
    for (int i = 0; i < kk; ++i) c[i] = -bot[i] > 0.0 ? -bot[i] : 0.0;
    PSDGB_CUDA_TRY(cudaMemcpyAsync(coef, c.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    PSDGB_CUDA_TRY(launch_rank_update(d_mat, n, Vb, coef, kk, s));
    return finish(ds, s);
}

psdgb_status check_deflate_args(double* d_mat, int64_t n, int64_t k, int maxiter) {
    if (n < 0 || k <= 0 || 3 * k > n || maxiter < 0 || (n > 0 && d_mat == nullptr) || n > 2147483647LL) {
        set_error("deflate: need a matrix, maxiter >= 0 and 0 < 3 k <= n (LOBPCG block, src/lobpcg.cu:25-27)");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    return PSDGB_OK;
}

}  // namespace

psdgb_status psdgb_eig_FP64_deflate(double* d_mat, int64_t n, int64_t k, int maxiter, double tol, uint64_t seed,
                                    void* stream) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    PSDGB_TRY(check_deflate_args(d_mat, n, k, maxiter));
    return deflate_two_ends(true, 0, 0, d_mat, n, k, maxiter, tol, seed, static_cast<cudaStream_t>(stream));
}

psdgb_status psdgb_composite_auto_scale_deflate_two_ends(int precision, int schedule, double* d_mat, int64_t n,
                                                         int64_t k, int maxiter, double tol, uint64_t seed,
                                                         void* stream) {
    std::lock_guard<std::recursive_mutex> call(g_call_mu);
    PrecisionInfo pi{};
    if (!precision_info(precision, &pi) || schedule_error(precision, schedule)) {
        set_error(std::string("composite deflate: ") +
                  (precision_info(precision, &pi) ? schedule_error(precision, schedule) : "unknown precision"));
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    PSDGB_TRY(check_deflate_args(d_mat, n, k, maxiter));
    return deflate_two_ends(false, precision, schedule, d_mat, n, k, maxiter, tol, seed,
                            static_cast<cudaStream_t>(stream));
}

uint64_t psdgb_kernel_launch_count(void) { return g_launches.load(); }

int psdgb_set_product_config(int acc_mode) {
    const int prev = g_single_acc_mode;
    if (acc_mode >= -1 && acc_mode <= ACC_1X4) g_single_acc_mode = acc_mode;
    return prev;
}

int psdgb_set_product_tuning(int knob, int value) {
    switch (knob) {
        case PSDGB_TUNE_TILE_GROUP: {
            const int prev = g_tile_group_rows;
            if (value >= 0 && value <= 64) g_tile_group_rows = value;
            return prev;
        }
        case PSDGB_TUNE_TILE_SHAPE: {
            const int prev = g_tile_shape;
            if (value >= -1 && value <= TILE_PAIR_256X256) g_tile_shape = value;
            return prev;
        }
        case PSDGB_TUNE_GROUP_EPI_WARPS: {
            const int prev = g_group_epi_warps;
            if (value == 4 || value == 8) g_group_epi_warps = value;
            return prev;
        }
        case PSDGB_TUNE_WIDE_KBLOCK: {
            const int prev = g_wide_kblock;
            if (value == 0 || value == 32 || value == 64) g_wide_kblock = value;
            return prev;
        }
        case PSDGB_TUNE_LANCZOS_SYMV: {
            const int prev = g_lanczos_symv;
            if (value >= -1 && value <= 2) g_lanczos_symv = value;
            return prev;
        }
        default: return -1;
    }
}

psdgb_status psdgb_product_timing_enable(int on) {
    product_timing_collect();
    std::lock_guard<std::mutex> lk(g_timing_mu);
    g_timing.on = on != 0;
    return PSDGB_OK;
}

psdgb_status psdgb_product_timing_read(double* ms, uint64_t* launches, double* mma_flops, int reset) {
    product_timing_collect();
    std::lock_guard<std::mutex> lk(g_timing_mu);
    if (ms) *ms = g_timing.ms;
    if (launches) *launches = g_timing.launches;
    if (mma_flops) *mma_flops = g_timing.flops;
    if (reset) {
        g_timing.ms = 0.0;
        g_timing.flops = 0.0;
        g_timing.launches = 0;
    }
    return PSDGB_OK;
}

psdgb_status psdgb_rel_frobenius(const double* d_a, const double* d_b, int64_t n, double* out, void* stream) {
    if (!out || n < 0) { set_error("bad arguments"); return PSDGB_ERR_INVALID_ARGUMENT; }
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* d2 = nullptr;
    PSDGB_CUDA_TRY(cudaMalloc(&d2, 2 * sizeof(double)));
    cudaError_t e = launch_diff_norms(d_a, d_b, n * n, d2, s);
    double h2[2] = {0.0, 0.0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h2, d2, sizeof(h2), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d2);
    if (e != cudaSuccess) return cuda_fail(e, "rel_frobenius");
    *out = h2[1] > 0.0 ? std::sqrt(h2[0] / h2[1]) : std::sqrt(h2[0]);
    return PSDGB_OK;
}

}  // extern "C"
