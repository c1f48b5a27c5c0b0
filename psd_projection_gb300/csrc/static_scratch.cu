// static_scratch.cu — psdgb_composite_static: the composite filter for
// callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc: a solver that reserves the GPU's memory
// up front and hands out only its own buffers, or a real-time loop that may
// not take the allocator's latency or failure modes.  psdgb_composite needs
// three operand matrices of scratch and, given no workspace, allocates it.
// This entry point instead uses one file-scope device array in this file's
// CUDA module, so a call allocates nothing.
//
// Limits and rules:
//   * n <= kStaticMaxN (512) and the FP16-split precisions only (PSDGB_PREC_FP16,
//     PSDGB_PREC_FP16X3): three 512 x 512 split matrices of two FP16 planes
//     (3 MiB) plus an error word.  Every GPU that loads the library holds
//     this array until the process exits.
//   * The first call on each device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current).  CUDA loads modules
//     lazily, so that lookup is also what loads the module holding the array,
//     which takes device memory once: make the first call before any stream
//     capture and before the caller reserves the GPU's memory.
//   * Every call shares the one array, and it keeps the last call's contents.
//     The operand matrices are fully rewritten by each call (padding included)
//     and the error word is cleared at the start of each call.  Calls that
//     overlap on the GPU (another thread, another stream) would race on the
//     array; calls from this library are serialised by a host lock and each
//     returns only after its stream has finished, also when it fails.
#include <mutex>
#include <string>

#include "internal.h"

namespace psdgb {
size_t composite_ws_bytes(int64_t n, int precision);
psdgb_status composite_run(DeviceState* ds, int precision, int schedule, double* mat, int64_t n, void* ws,
                           bool auto_scale, int64_t max_iter, double tol, uint64_t seed, int residual_mode,
                           void* lz_state, cudaStream_t s, double* up_out);
}  // namespace psdgb

namespace {

constexpr int64_t kStaticMaxN = 512;
// Three FP16 split matrices (hi and lo planes) of kStaticMaxN^2 elements.
constexpr size_t kStaticOperandBytes = 3u * 2u * 2u * kStaticMaxN * kStaticMaxN;
constexpr size_t kStaticBytes = kStaticOperandBytes + 256;  // + the error word

// The scratch.  In host code this name is only a stand-in for the device
// object: never pass it to a kernel; use the address from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

constexpr int kMaxDevices = 64;
char* g_scratch_addr[kMaxDevices] = {};  // device address of g_static_scratch, per device
std::mutex g_static_mu;                 // one call at a time uses the array

// Per-device set-up: the array's device address, looked up with the device current.
psdgb_status scratch_for_device(int dev, char** out) {
    if (dev < 0 || dev >= kMaxDevices) {
        psdgb::set_error("psdgb_composite_static: device index out of range");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (g_scratch_addr[dev] == nullptr) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return psdgb::cuda_fail(e, "cudaGetSymbolAddress(g_static_scratch)");
        g_scratch_addr[dev] = static_cast<char*>(p);
    }
    *out = g_scratch_addr[dev];
    return PSDGB_OK;
}

}  // namespace

extern "C" psdgb_status psdgb_composite_static(int precision, int schedule, double* d_mat, int64_t n,
                                               void* stream) {
    using namespace psdgb;
    if (precision != PSDGB_PREC_FP16 && precision != PSDGB_PREC_FP16X3) {
        set_error("psdgb_composite_static supports PSDGB_PREC_FP16 and PSDGB_PREC_FP16X3 only");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (n < 0 || n > kStaticMaxN) {
        set_error("psdgb_composite_static: n = " + std::to_string(n) + " is outside [0, " +
                  std::to_string(kStaticMaxN) + "], the size of its static scratch");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (n > 0 && d_mat == nullptr) {
        set_error("null matrix");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return PSDGB_OK;
    if (composite_ws_bytes(n, precision) > kStaticOperandBytes) {
        set_error("psdgb_composite_static: operands do not fit the static scratch");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(g_static_mu);
    DeviceState ds;
    PSDGB_CUDA_TRY(cudaGetDevice(&ds.device));
    PSDGB_CUDA_TRY(cudaDeviceGetAttribute(&ds.cc_major, cudaDevAttrComputeCapabilityMajor, ds.device));
    PSDGB_CUDA_TRY(cudaDeviceGetAttribute(&ds.cc_minor, cudaDevAttrComputeCapabilityMinor, ds.device));
    PSDGB_CUDA_TRY(cudaDeviceGetAttribute(&ds.sm_count, cudaDevAttrMultiProcessorCount, ds.device));
    if (!(ds.cc_major == 10 && ds.cc_minor == 3)) {
        set_error("psdgb kernels are built for sm_103a");
        return PSDGB_ERR_UNSUPPORTED;
    }
    char* scratch = nullptr;
    PSDGB_TRY(scratch_for_device(ds.device, &scratch));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ds.d_error = reinterpret_cast<int*>(scratch + kStaticOperandBytes);
    PSDGB_CUDA_TRY(cudaMemsetAsync(ds.d_error, 0, sizeof(int), s));
    const psdgb_status st =
        composite_run(&ds, precision, schedule, d_mat, n, scratch, false, 0, 0.0, 0, 0, nullptr, s, nullptr);
    if (st != PSDGB_OK) {
        // Work queued before the failure may still use the array: wait for it
        // before the lock lets another call in.  The first error is the one reported.
        cudaStreamSynchronize(s);
        cudaGetLastError();
        return st;
    }
    return finish(&ds, s);
}
