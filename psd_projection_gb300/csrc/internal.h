// internal.h — host-side declarations shared by the psdgb translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <cuda.h>
#include <cuda_runtime.h>

#include "common.cuh"
#include "psdgb.h"

namespace psdgb {

// ---- error reporting (capi.cu) ----------------------------------------------
void set_error(const std::string& msg);
psdgb_status cuda_fail(cudaError_t e, const char* what);
void count_launch(uint64_t k = 1);

#define PSDGB_CUDA_TRY(expr)                                      \
    do {                                                          \
        cudaError_t _e = (expr);                                  \
        if (_e != cudaSuccess) return ::psdgb::cuda_fail(_e, #expr); \
    } while (0)

#define PSDGB_TRY(expr)                           \
    do {                                          \
        psdgb_status _s = (expr);                 \
        if (_s != PSDGB_OK) return _s;            \
    } while (0)

// Per-device state: a small device buffer holding the error word of the
// bounded waits, plus cached workspaces.
struct DeviceState {
    int device = -1;
    int* d_error = nullptr;  // device error word (DeviceError)
    void* ws = nullptr;      // cached composite workspace
    size_t ws_bytes = 0;
    void* lz = nullptr;      // cached Lanczos state
    size_t lz_bytes = 0;
    int sm_count = 0;
    int cc_major = 0, cc_minor = 0;
    // Host-sequence projections (psdgb_project_host_many): copy streams,
    // ordering events and kHostStages staging matrices, created on first use.
    static constexpr int kHostStages = 3;
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaEvent_t in_done[kHostStages] = {}, comp_done[kHostStages] = {}, out_done[kHostStages] = {};
    void* stage2 = nullptr;
    size_t stage2_bytes = 0;
};
psdgb_status device_state(DeviceState** out);
// Upper bound on the CTAs (one per SM) of the persistent kernels this thread
// launches, 0 for every SM: the request loop caps its large requests' kernels
// so that some SMs stay free for small requests (csrc/serve.cu).
extern thread_local int g_sm_cap;
inline int sm_budget(const DeviceState* ds) {
    return (g_sm_cap > 0 && g_sm_cap < ds->sm_count) ? g_sm_cap : ds->sm_count;
}
// Synchronise the stream and turn a device error word into a status.
psdgb_status finish(DeviceState* ds, cudaStream_t stream);

// FP32 row-major matrix of rows x cols (row stride ld elements, a multiple of
// 4) as a TMA tensor map of unswizzled box_rows x box_cols tiles, zero fill
// outside the matrix (gemm_tc.cu).
bool make_tmap_f32(CUtensorMap* tm, const void* base, int64_t ld, int64_t rows, int64_t cols, int box_rows,
                   int box_cols);

// ---- product timing (capi.cu) --------------------------------------------------
// Record an event before / after a product launch when timing is enabled.
void product_timing_begin(cudaStream_t s);
void product_timing_end(cudaStream_t s, double mma_flops);
// Fold the finished event pairs into the totals (after a stream sync).
void product_timing_collect();

// ---- precision helpers (composite.cu) -------------------------------------------
struct PrecisionInfo {
    int fmt;        // storage Format of the operands
    int nprod;      // products per term pair list (1, 3, 6, 9); 0 for SIMT
    int terms;      // operand terms read by the products
};
bool precision_info(int precision, PrecisionInfo* out);
inline int64_t pad128(int64_t n) { return (n + 127) / 128 * 128; }
// Whether a precision may run a schedule (nullptr) or why not.  One-term BF16
// operands round eigenvalues past 1 where the FP32 table's last two steps have
// no safety factor, and the quintic diverges: BF16 needs a factor on every
// step.  E4M3 operands (2^-4 rounding) diverge even with the FP16 table's
// 1.01: FP8 runs the FP8 schedule.
inline const char* schedule_error(int precision, int schedule) {
    if (schedule != PSDGB_SCHEDULE_FP32 && schedule != PSDGB_SCHEDULE_FP16 && schedule != PSDGB_SCHEDULE_FP8)
        return "unknown schedule";
    if (precision == PSDGB_PREC_FP8 && schedule != PSDGB_SCHEDULE_FP8)
        return "FP8 products need the FP8 schedule (safety factor 1.5 on every step)";
    if (precision == PSDGB_PREC_BF16 && schedule == PSDGB_SCHEDULE_FP32)
        return "one-term BF16 products need the FP16 schedule (safety factor on every step)";
    return nullptr;
}
size_t split_matrix_bytes(int fmt, int64_t np);

// ---- elementwise kernels (elem.cu) --------------------------------------------
// a32 (n x ld, ld = pad4(n), zero padded) = FP32 of the symmetric matrix
// defined by the upper triangle of the column-major FP64 matrix x.
cudaError_t launch_sym_upper_to_f32(const double* x, int64_t n, float* a32, int64_t ld, cudaStream_t s);
// out (Np x Np split matrix) = split(scale * (*scale_dev) * a32), zero padding
// (scale_dev may be null: factor 1).
// FP32 input variants: the FP32 copy of a column-major FP32 matrix's upper
// triangle, and the split of it (scaled) into operand terms.
cudaError_t launch_sym_upper_f32_to_f32(const float* x, int64_t n, float* a32, int64_t ld, cudaStream_t s);
cudaError_t launch_split_from_f32_upper(const float* x, int64_t n, double scale, const double* scale_dev,
                                        const SplitMat& out, int fmt, int64_t np, cudaStream_t s);
cudaError_t launch_split_from_f32(const float* a32, int64_t n, int64_t ld, double scale, const double* scale_dev,
                                  const SplitMat& out, int fmt, int64_t np, cudaStream_t s);
// out (Np x Np split matrix) = split(scale * (*scale_dev) * sym_upper(x)), zero padding.
cudaError_t launch_split_from_f64_upper(const double* x, int64_t n, double scale, const double* scale_dev,
                                        const SplitMat& out, int fmt, int64_t np, cudaStream_t s);
// FP64 reductions: out[0] = sum (a-b)^2, out[1] = sum b^2 over n*n elements.
cudaError_t launch_diff_norms(const double* a, const double* b, int64_t count, double* d_out2, cudaStream_t s);
// Scale column j of v (n x n col-major FP64) by max(w[j], 0).
cudaError_t launch_scale_columns_relu(double* v, const double* w, int64_t n, cudaStream_t s);
cudaError_t launch_scale_columns_relu_f32(float* v, const float* w, int64_t n, cudaStream_t s);
cudaError_t launch_f64_to_f32(const double* in, float* out, int64_t count, cudaStream_t s);
cudaError_t launch_f32_to_f64(const float* in, double* out, int64_t count, cudaStream_t s);

// ---- symmetric products (gemm_simt.cu, gemm_tc.cu) -----------------------------
// C = P * Q for symmetric P, Q (Np x Np split matrices); the epilogue ep
// consumes C.  precision selects the kernel and the term products.
psdgb_status gemm_symmetric(DeviceState* ds, int precision, const SplitMat& P, const SplitMat& Q, int64_t np,
                            const EpiParams& ep, cudaStream_t s);
psdgb_status gemm_simt(DeviceState* ds, const SplitMat& P, const SplitMat& Q, int64_t np, const EpiParams& ep,
                       cudaStream_t s);
psdgb_status gemm_tc(DeviceState* ds, int precision, const SplitMat& P, const SplitMat& Q, int64_t np,
                     const EpiParams& ep, cudaStream_t s);
// Accumulator configurations of the tensor-core product kernel: ACC_SPLIT
// interleaved accumulators (K/ACC_SPLIT additions each) x ACC_BUFS sets
// (epilogue of one tile overlapping the next tile's MMAs); 512 TMEM columns.
enum AccMode : int { ACC_4X1 = 0, ACC_2X2 = 1, ACC_1X4 = 2 };
extern int g_single_acc_mode;  // forced configuration of single-matrix products, or -1 (automatic)
int auto_acc_mode(int precision, int64_t np);
// Tile shape of single-matrix products: one CTA per 128 x 128 tile (gemm_tc.cu),
// a CTA pair per 256 x 128 tile (gemm_tc2.cu), one CTA per 128 x 256 tile
// (gemm_wide.cu; one- and two-term precisions, others use 128 x 128), a CTA
// pair per 256 x 256 tile (gemm_pairwide.cu; one- and two-term precisions);
// -1 chooses: 256 x 256 pairs for one- and two-term precisions at np >= 2048.
enum TileShape : int { TILE_128X128 = 0, TILE_PAIR_256X128 = 1, TILE_WIDE_128X256 = 2, TILE_PAIR_256X256 = 3 };
extern int g_tile_shape;
extern int g_group_epi_warps;  // epilogue warps of 128 x 128 tiles with four accumulator buffers: 4 or 8
extern int g_wide_kblock;  // K block of the 128 x 256 kernel: 64, 32, or 0 (by precision)
extern int g_tile_group_rows;  // tile order of single-matrix products (grouped_decode), 0 = row by row
extern int g_lanczos_symv;  // Lanczos matvec over 128 x 128 triangle tiles: -1 automatic (n >= 2048), 0 off, 1 on
// One matrix on CTA pairs (gemm_tc2.cu): 256 x 128 tiles, one
// tcgen05.mma.cta_group::2 per term product and K slice; np >= 256.
psdgb_status gemm_tc_pair(DeviceState* ds, int precision, int acc_mode, const SplitMat& P, const SplitMat& Q,
                          int64_t np, const EpiParams& ep, cudaStream_t s);
// One matrix on CTA pairs with 256 x 256 tiles (gemm_pairwide.cu): one- and two-term precisions.
psdgb_status gemm_tc_pairwide(DeviceState* ds, int precision, const SplitMat& P, const SplitMat& Q, int64_t np,
                              const EpiParams& ep, cudaStream_t s);
// The batch's pair tiles (TileDesc {block, I, J}: the 256 x 256 tile of tile
// rows 2I, 2I + 1 against 2J, 2J + 1 of that block, both rows inside it) on
// the same kernel; operands in the strided layout (ld, rows).
bool pairwide_supported(int precision);
psdgb_status gemm_tc_pairwide_group(DeviceState* ds, int precision, const SplitMat& P, const SplitMat& Q, int64_t ld,
                                    int64_t rows, const EpiParams& ep, const GroupWork& gw, int64_t num_pairs,
                                    cudaStream_t s);
// One matrix on 128 x 256 tiles (gemm_wide.cu): one- and two-term precisions; np >= 256.
psdgb_status gemm_tc_wide(DeviceState* ds, int precision, const SplitMat& P, const SplitMat& Q, int64_t np,
                          const EpiParams& ep, cudaStream_t s);
// Grouped product over a tile list (see GroupWork), persistent over `grid`
// CTAs (0: one per SM); operand planes of `rows` rows with row stride ld.
psdgb_status gemm_tc_group(DeviceState* ds, int precision, int acc_mode, const SplitMat& P, const SplitMat& Q,
                           int64_t ld, int64_t rows, const EpiParams& ep, const GroupWork& gw, int64_t num_tiles,
                           int grid, cudaStream_t s);

// ---- small blocks of a batch, whole chain on chip (batch_chain.cu) ---------------
// One block of n <= 128 for batch_chain_kernel: its FP32 copy (rows of ld4
// floats) and bound (scale = up or 1, and its inverse) from the batch's
// Lanczos launch, and its offset in the packed FP64 blocks.
struct ChainBlock {
    const float* a32;
    int ld4;
    int n;
    long long x_off;
    const double* scale;
    const double* inv_scale;
};
// The split, the steps' products and the final reconstruction of `count`
// such blocks (FP16 / FP16x3), one persistent launch of `grid` CTAs (0: one
// per SM) that claim blocks from *d_counter (reset on stream s first).
psdgb_status launch_batch_chain(DeviceState* ds, int precision, const ChainBlock* d_blocks, int count,
                                const float* coef, int steps, double* d_x, int* d_counter, int grid,
                                cudaStream_t s);

// ---- Lanczos (lanczos.cu) ---------------------------------------------------------
struct LanczosResult {
    double lo = 0.0, up = 1.0, theta = 0.0;
    int64_t nb_iter = 0;
};
size_t lanczos_state_bytes(int64_t n, int64_t max_iter);
// Enqueue the whole bound on a32 (n x ld FP32, symmetric) on stream s; the
// results stay in the device state.  d_warm (n doubles, may be null) replaces
// the seeded start vector; d_ritz_out (n doubles, may be null) receives the
// Ritz vector.  No host synchronisation.
psdgb_status lanczos_bound_async(DeviceState* ds, const float* a32, int64_t n, int64_t ld, int64_t max_iter,
                                 double tol, uint64_t seed, int residual_mode, void* d_state, cudaStream_t s,
                                 const double* d_warm, double* d_ritz_out);
// Device addresses of the scale (up, or 1) and of its inverse in the state.
const double* lanczos_scale_ptr(void* d_state, int64_t n, int64_t max_iter);
const double* lanczos_inv_scale_ptr(void* d_state, int64_t n, int64_t max_iter);
// Copy the bound (and alpha/beta when non-null) to the host; synchronises s.
psdgb_status lanczos_read(void* d_state, int64_t n, int64_t max_iter, cudaStream_t s, LanczosResult* res,
                          double* h_alpha, double* h_beta);

// ---- shared by the entry points (capi.cu, composite.cu, eigenpairs.cu) --------
size_t composite_ws_bytes(int64_t n, int precision);
psdgb_status composite_enqueue(DeviceState* ds, int precision, int schedule, double* mat, int64_t n, void* ws,
                               bool auto_scale, int64_t max_iter, double tol, uint64_t seed, int residual_mode,
                               void* lz_state, cudaStream_t s, const double* d_warm, double* d_ritz_out,
                               int bulk_precision, int refine_steps);
psdgb_status composite_enqueue_scaled(DeviceState* ds, int precision, int schedule, double* mat, int64_t n, void* ws,
                                      double scale, cudaStream_t s);
psdgb_status composite_enqueue_f32(DeviceState* ds, int precision, int schedule, float* mat, int64_t n, void* ws,
                                   int64_t max_iter, double tol, uint64_t seed, int residual_mode, void* lz_state,
                                   cudaStream_t s, const double* d_warm, double* d_ritz_out);

// ---- eigenpairs and deflation (eigenpairs.cu) -----------------------------------
// X += sum_i coef_i v_i v_i^T (column-major n x n; V n x r column-major; coef on the device).
cudaError_t launch_rank_update(double* X, int64_t n, const double* V, const double* d_coef, int r, cudaStream_t s);
// One wait on a barrier nothing arrives at, bounded by limit_ns (elem.cu).
cudaError_t launch_wait_selftest(int* err, uint64_t limit_ns, cudaStream_t s);
// x[i] *= a, i < count (lobpcg.cu).
cudaError_t launch_scale_inplace(double* x, int64_t count, double a, cudaStream_t s);
}  // namespace psdgb
