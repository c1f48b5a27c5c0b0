/*
 * psdgb.h — C ABI of the GB300-native PSD-cone projection library (libpsdgb.so).
 *
 * Every entry point takes plain pointers and sizes.  Device matrices are n x n
 * FP64, column-major, leading dimension n, exactly as the reference library's
 * `double* mat` arguments.  The matrix is assumed symmetric; where it is not,
 * the library uses the symmetric matrix defined by its upper triangle
 * (row <= column), the same triangle cuSOLVER syevd reads in eig_FP64_psd.
 *
 * All calls are blocking on the given stream (they end with a stream
 * synchronisation), like the reference functions, which end in
 * cudaDeviceSynchronize.  Unlike the reference (whose CHECK_* macros print and
 * continue, include/psd_projection/check.h:18-57), every call returns a status
 * code; psdgb_last_error() gives the message of the last failure on the
 * calling thread.
 *
 * Reference interfaces replaced (paths inside ComputationalRobotics/psd_projection):
 *   psdgb_composite            composite_FP16 / composite_FP32 / composite_FP32_emulated
 *                              (include/psd_projection/composite_FP16.h:12-18,
 *                               composite_FP32.h:12-17, composite_FP32_emulated.h:17-22)
 *   psdgb_composite_auto_scale composite_*_auto_scale
 *                              (composite_FP16.h:26-33, composite_FP32.h:24-30,
 *                               composite_FP32_emulated.h:29-35)
 *   psdgb_two_norm             approximate_two_norm (include/psd_projection/lanczos.h:11-17)
 *   psdgb_eig_psd              eig_FP64_psd / eig_FP32_psd
 *                              (include/psd_projection/eig_FP64_psd.h:14-20, eig_FP32_psd.h:14-20)
 *   psdgb_project              the MATLAB wrapper's method dispatch
 *                              (MATLAB/psd_projection_MATLAB.cu:62-188), device buffers
 *   psdgb_project_host         the same dispatch on host buffers, with the H2D/D2H copies
 *                              of MATLAB/psd_projection_MATLAB.cu:104-106,171-173
 */
#ifndef PSDGB_H
#define PSDGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum psdgb_status {
    PSDGB_OK = 0,
    PSDGB_ERR_INVALID_ARGUMENT = 1, /* bad size, null pointer, unknown method/precision */
    PSDGB_ERR_CUDA = 2,             /* a CUDA runtime call or a kernel launch failed */
    PSDGB_ERR_OUT_OF_MEMORY = 3,    /* internal workspace could not be allocated */
    PSDGB_ERR_UNSUPPORTED = 4,      /* device is not sm_103 (the kernels are sm_103a only) */
    PSDGB_ERR_DEVICE_TIMEOUT = 5,   /* a bounded device-side wait gave up (error flag set) */
    PSDGB_ERR_SOLVER = 6,           /* cuSOLVER reported a failure (eig_* entry points) */
    PSDGB_ERR_WORKSPACE_TOO_SMALL = 7
} psdgb_status;

/* Operand arithmetic of the filter's matrix products.  Every mode accumulates
 * in FP32; the elementwise polynomial combination is done in FP32. */
typedef enum psdgb_precision {
    PSDGB_PREC_FP32_SIMT = 0, /* plain FP32 FMA on the CUDA cores (the reference's Sgemm numerics) */
    PSDGB_PREC_FP16 = 1,      /* one FP16 term per operand, tcgen05 kind::f16 */
    PSDGB_PREC_BF16 = 2,      /* one BF16 term per operand */
    PSDGB_PREC_FP16X3 = 3,    /* FP16 hi/lo split, products hi*hi + hi*lo + lo*hi */
    PSDGB_PREC_BF16X3 = 4,    /* BF16 hi/lo split, 3 products */
    PSDGB_PREC_BF16X6 = 5,    /* BF16 3-term split, the 6 products of order <= 2 */
    PSDGB_PREC_BF16X9 = 6,    /* BF16 3-term split, all 9 products (FP32 emulation) */
    PSDGB_PREC_FP8 = 7        /* one FP8 E4M3 term per operand, tcgen05 kind::f8f6f4, FP32 accumulate;
                                 the stored iterate keeps the FP16 hi/lo pair (FP16 schedule only) */
} psdgb_precision;

/* Polynomial schedule of the sign filter. */
typedef enum psdgb_schedule {
    PSDGB_SCHEDULE_FP32 = 0,  /* 10 quintic steps, safety factor 1.001 on the first 8
                                 (src/composite_FP32.cu:73-99) */
    PSDGB_SCHEDULE_FP16 = 1,  /* 7 quintic steps, safety factor 1.01 on every step
                                 (src/composite_FP16.cu:93-113) */
    PSDGB_SCHEDULE_FP8 = 2    /* the FP16 table's 7 steps with safety factor 1.5 on every step: E4M3
                                 operand rounding (2^-4) pushes eigenvalues well past 1.01 (no
                                 counterpart in the reference; the schedule of PSDGB_PREC_FP8) */
} psdgb_schedule;

/* Residual formula of the Lanczos upper bound. */
typedef enum psdgb_residual {
    PSDGB_RESIDUAL_REFERENCE = 0, /* r = A*y - theta*y, what src/lanczos.cu:246-260 computes
                                     (its copy at :255 leaves ry = A*y) */
    PSDGB_RESIDUAL_EXACT = 1      /* r = A^T*A*y - theta*y, the Ritz residual of A^T*A */
} psdgb_residual;

/* ---- library information ------------------------------------------------ */
int psdgb_version(void);
const char* psdgb_last_error(void);
/* Host-side name of a precision/schedule enum value, or NULL. */
const char* psdgb_precision_name(int precision);

/* Per-step coefficients (a, b, c) of a filter schedule after the safety
 * scaling p(x/s), as FP32 triples in out[3*i .. 3*i+2].  Writes at most cap
 * triples and returns the number of steps, or -1 for an unknown schedule. */
int psdgb_filter_coefficients(int schedule, float* out, int cap);

/* ---- workspace -------------------------------------------------------------
 * Bytes of device workspace psdgb_composite / psdgb_composite_auto_scale need
 * for the filter operands of an n x n matrix at the given precision (three
 * split matrices of Np x Np, Np = n rounded up to 128).  A caller that passes
 * ws == NULL, or ws_bytes below this size, gets the library's own cached
 * workspace (allocated on first use, grown on demand and kept until
 * psdgb_release_workspace or process exit).  The Lanczos state (a few
 * n-vectors and the n x max_iter basis) always comes from a cached buffer.
 * A caller workspace (and a caller Lanczos state) must be 16-byte aligned
 * (cudaMalloc gives 256): the kernels read it through TMA tensor maps and
 * 16-byte vectors; an unaligned one is refused with
 * PSDGB_ERR_INVALID_ARGUMENT before any work is enqueued. */
size_t psdgb_composite_workspace_size(int64_t n, int precision);
psdgb_status psdgb_release_workspace(void);

/* ---- the hot path ---------------------------------------------------------- */

/* Composite polynomial filter on a matrix whose spectrum lies in [-1, 1]
 * (composite_FP16 / composite_FP32 / composite_FP32_emulated).  In place. */
psdgb_status psdgb_composite(int precision, int schedule, double* d_mat, int64_t n,
                             void* d_ws, size_t ws_bytes, void* stream);

/* psdgb_composite for callers that cannot allocate device memory: a solver
 * that reserves the GPU's memory up front and hands out only its own buffers,
 * or a real-time loop that may not wait on, or fail in, the allocator.  The
 * operand scratch is a file-scope device array inside this library's CUDA
 * module, so the call allocates nothing.  No counterpart in the reference.
 * Limits: precision PSDGB_PREC_FP16 or PSDGB_PREC_FP16X3 and n <= 512 (the
 * array is 3 MiB, held on every GPU that loads the library until exit);
 * larger n returns PSDGB_ERR_INVALID_ARGUMENT.  The first call on a device
 * does the set-up: it looks up the array's device address, and (CUDA loads
 * modules lazily) that lookup loads the module that holds the array, which
 * takes device memory once.  Make that first call before any stream capture
 * and before reserving the GPU's memory.  All calls share the array, which
 * keeps the last call's contents: calls that overlap on the GPU race on it
 * (this library serialises its own calls; each waits for its stream before
 * returning, on the error path too). */
psdgb_status psdgb_composite_static(int precision, int schedule, double* d_mat, int64_t n, void* stream);

/* Lanczos bound, scale by 1/up, filter, and rescale by up
 * (composite_*_auto_scale).  max_iter = 20 and tol = 1e-10 are the
 * reference's defaults (src/composite_FP32.cu:177-179 uses the defaults of
 * lanczos.h:16).  seed selects the start vector.  up_out may be NULL. */
psdgb_status psdgb_composite_auto_scale(int precision, int schedule, double* d_mat, int64_t n,
                                        int64_t lanczos_max_iter, double lanczos_tol,
                                        uint64_t seed, int residual_mode,
                                        void* d_ws, size_t ws_bytes, void* stream,
                                        double* up_out);

/* Bytes of the Lanczos state (a few n-vectors, the n x max_iter basis, the
 * tridiagonal solver's scratch and, for the triangle-tile matvec, the FP64
 * partial sums: n^2 / 16 bytes). */
size_t psdgb_lanczos_state_size(int64_t n, int64_t max_iter);

/* psdgb_composite_auto_scale without any host synchronisation: the Lanczos
 * bound, the scale 1/up and the filter are enqueued on `stream` and the call
 * returns.  Nothing is allocated: the caller provides the filter workspace
 * (>= psdgb_composite_workspace_size) and the Lanczos state
 * (>= psdgb_lanczos_state_size) and must not reuse either, or read d_mat,
 * before the stream has passed this work.  d_warm_start (n doubles, device,
 * may be NULL) replaces the seeded start vector — e.g. the previous Ritz
 * vector of a slowly changing matrix; d_ritz_out (n doubles, may be NULL)
 * receives this call's Ritz vector.  A bounded device wait that gives up is
 * reported by the next psdgb_check_device_error() (or synchronous call).
 * The enqueued work can be captured in a CUDA graph. */
psdgb_status psdgb_composite_auto_scale_async(int precision, int schedule, double* d_mat, int64_t n,
                                              int64_t max_iter, double tol, uint64_t seed, int residual_mode,
                                              const double* d_warm_start, double* d_ritz_out,
                                              void* d_ws, size_t ws_bytes, void* d_lanczos,
                                              size_t lanczos_bytes, void* stream);

/* The auto-scaled projection of an FP32 matrix, in place, for callers whose
 * iterate is FP32 (an ADMM loop): d_mat is n x n column-major FP32 on the
 * device and its upper triangle defines it.  The Lanczos bound streams an
 * FP32 copy as in the FP64 path, the filter runs at `precision` (a
 * tensor-core precision), and the final reconstruction computes in FP64 and
 * writes FP32: the FP64 path's result rounded to FP32, with half its HBM and
 * host-copy traffic.  Warm start / Ritz output as in
 * psdgb_composite_auto_scale_async.  Asynchronous (no host synchronisation)
 * when the caller passes both workspaces; d_ws / d_lanczos may be null or too
 * small, and the library's cached buffers are then used and the call waits
 * for its stream before returning, so later calls can reuse those buffers. */
psdgb_status psdgb_composite_auto_scale_f32(int precision, int schedule, float* d_mat, int64_t n, int64_t max_iter,
                                            double tol, uint64_t seed, int residual_mode, const double* d_warm_start,
                                            double* d_ritz_out, void* d_ws, size_t ws_bytes, void* d_lanczos,
                                            size_t lanczos_bytes, void* stream);

/* Mixed precision (no counterpart in the reference): the Lanczos bound, the
 * bulk_schedule's steps with bulk_precision products (one-term FP16 or BF16),
 * then refine_steps steps of the quintic that ends the FP32 table (no safety
 * factor) and the final reconstruction with refine_precision products
 * (fp16x3 after fp16; bf16x3/x6/x9 after bf16 — the same operand format). */
psdgb_status psdgb_composite_mixed_auto_scale(int bulk_precision, int bulk_schedule, int refine_precision,
                                              int refine_steps, double* d_mat, int64_t n, void* stream);

/* Synchronise the device and report (and clear) a device-side wait failure. */
psdgb_status psdgb_check_device_error(void);

/* Lanczos spectral-norm bound (approximate_two_norm): lo and up are host
 * pointers.  The matrix is not modified. */
psdgb_status psdgb_two_norm(const double* d_A, int64_t n, double* lo, double* up,
                            int64_t max_iter, double tol, uint64_t seed, int residual_mode,
                            void* d_ws, size_t ws_bytes, void* stream);

/* Diagnostic variant of psdgb_two_norm: also returns the Lanczos coefficients
 * (alpha, beta: host arrays of max_iter doubles, may be NULL), the number of
 * completed iterations and the Ritz value theta. */
psdgb_status psdgb_two_norm_ex(const double* d_A, int64_t n, double* lo, double* up,
                               int64_t max_iter, double tol, uint64_t seed, int residual_mode,
                               void* d_ws, size_t ws_bytes, void* stream,
                               double* h_alpha, double* h_beta, int64_t* nb_iter,
                               double* theta);

/* EVD projection through cuSOLVER syevd (eig_FP64_psd when fp64 != 0, else
 * eig_FP32_psd).  When d_eigs_out is not NULL it receives the n unclipped
 * eigenvalues in ascending order (FP64, device), which the reference returns
 * as a library-allocated pointer. */
psdgb_status psdgb_eig_psd(int fp64, double* d_mat, int64_t n, double* d_eigs_out, void* stream);

/* Method-string dispatch of the MATLAB wrapper: "composite_FP16",
 * "composite_FP32", "composite_FP32_emulated", "eig_FP64", "eig_FP32".  The
 * composite methods run the Lanczos bound with the reference defaults.  For
 * eig_* methods d_eigs_out (n doubles, may be NULL) gets the eigenvalues. */
psdgb_status psdgb_project(const char* method, double* d_mat, int64_t n, double* d_eigs_out,
                           void* stream);

/* psdgb_project on host buffers: copies h_in to the device, projects, and
 * copies the result to h_out (h_out may equal h_in).  h_eigs_out (n doubles,
 * host) may be NULL.  Pinned host buffers give the fastest copies. */
psdgb_status psdgb_project_host(const char* method, const double* h_in, double* h_out,
                                int64_t n, double* h_eigs_out, void* stream);

/* ---- request loop (continuous batching of mixed-size projections) ---------- */
/* No counterpart in the reference (its calls block and allocate per call).
 * An ADMM-style caller submits projections of device matrices tagged by a
 * key (one ADMM stream); the server runs up to max_slots of them at once,
 * each on its own CUDA stream with private buffers, admits queued requests as
 * slots and HBM budget free up, keeps each key's last Ritz vector on the
 * device and warm-starts the key's next Lanczos bound from it, and can replay
 * one captured CUDA graph per (slot, n).  Requests of one key run in
 * submission order.  Single host thread. */
typedef struct psdgb_server psdgb_server;

typedef struct psdgb_server_config {
    size_t hbm_budget_bytes;  /* device bytes the server may hold (slot buffers, warm starts) */
    int max_slots;            /* requests in flight at once (1..256) */
    int precision;            /* psdgb_precision (tensor-core modes) */
    int schedule;             /* psdgb_schedule */
    int64_t max_iter;         /* Lanczos steps from the seeded start (reference default 20) */
    int64_t warm_max_iter;    /* Lanczos steps from a key's previous Ritz vector */
    int use_graphs;           /* capture each (slot, n) projection once and replay it */
    int admission;            /* PSDGB_ADMIT_FIFO: queued requests start in submission order (a request
                                 that does not fit the budget yet is skipped); PSDGB_ADMIT_SHORTEST_FIRST:
                                 among each key's oldest queued request, the smallest n starts first
                                 (ties by submission).  Both keep every key's requests in order. */
    int64_t priority_n;       /* > 0: requests with n <= priority_n run on high-priority streams and the
                                 persistent kernels of larger requests leave reserve_sms SMs free; 0: off */
    int reserve_sms;          /* SMs kept free of large requests' persistent kernels (with priority_n) */
    int reserve_slots;        /* slots large requests may not take (with priority_n; < max_slots) */
} psdgb_server_config;
enum { PSDGB_ADMIT_FIFO = 0, PSDGB_ADMIT_SHORTEST_FIRST = 1 };

typedef struct psdgb_completion {
    uint64_t ticket;
    int64_t key;
    int64_t n;
    int status;               /* psdgb_status of the request */
    double submit_s;          /* psdgb_clock_seconds() at submission */
    double start_s;           /* ... when the request was admitted to a slot */
    double end_s;             /* ... when poll saw it finished */
    double gpu_ms;            /* device time from admission to completion (CUDA events) */
} psdgb_completion;

double psdgb_clock_seconds(void);
psdgb_status psdgb_server_create(const psdgb_server_config* cfg, psdgb_server** out);
psdgb_status psdgb_server_destroy(psdgb_server* server);
/* Queue the projection of d_in (n x n FP64, device; read when the request
 * starts) into d_out (device, may equal d_in). */
psdgb_status psdgb_server_submit(psdgb_server* server, int64_t key, const double* d_in, double* d_out, int64_t n,
                                 uint64_t* ticket);
/* Retire finished requests into out[0..cap) (*n_out of them) and admit queued
 * ones; with wait != 0, block until at least one request finishes. */
psdgb_status psdgb_server_poll(psdgb_server* server, int wait, psdgb_completion* out, int cap, int* n_out);
psdgb_status psdgb_server_stats(psdgb_server* server, int* in_flight, int* queued, size_t* bytes_used,
                                uint64_t* completed);

/* ---- block-diagonal batches ---------------------------------------------------
 * No counterpart in the reference, which projects one matrix per call.  A plan
 * for `count` symmetric blocks of the given sizes (0..4096) projects all of
 * them with about 40 kernel launches (independent of count): one CTA per
 * block for the Lanczos bound, one persistent tensor-core kernel per product
 * over the tiles of every block.  The blocks are packed column-major, one after the
 * other (block b starts at element sum_{c<b} n_c^2), and projected in place —
 * the layout of a block-diagonal SDP iterate.  psdgb_batch_project is
 * asynchronous and allocates nothing (the plan owns its device memory), so
 * it can be captured in a CUDA graph; a plan serves one projection at a time
 * (its operand buffers are per plan): make one plan per concurrent stream.
 *
 * With FP16 / FP16x3 operands the blocks of n <= 128 (one 128 x 128 tile)
 * can instead run their whole filter in one persistent kernel that keeps
 * their three split matrices in shared memory ("small blocks on chip", the
 * default for such plans); the per-product launches then take only the
 * larger blocks.  Both routes give the same result bit for bit when the
 * products use one accumulator per tile (acc_mode 2).
 *
 * Tile shape: the products of blocks of n > 128 run on 128 x 128 tiles (the
 * default), or (pair_tiles = 1, where the precision allows it) on 256 x 256
 * tiles shared by a pair of SMs wherever two tile rows of a block fit (the
 * odd last tile row of a block stays on 128 x 128 tiles): half the operand
 * bytes per multiply-add.
 *
 * Serpentine order (serpentine = 1): every other product walks its tile lists
 * backwards, so that it starts on the blocks whose operands the product
 * before it left in L2.
 *
 * psdgb_batch_autotune times every tile shape, accumulator configuration,
 * tile order and (where available) the on-chip route on the caller's scratch
 * blocks (overwritten) and keeps the fastest; the serpentine order stays as
 * configured (off by default).
 * psdgb_batch_configure sets them by hand (-1 keeps a setting; acc_mode
 * 0..2, tile_order 0 (largest blocks first) or 1 (block order),
 * small_on_chip, pair_tiles and serpentine 0 or 1 — small_on_chip or
 * pair_tiles 1 is refused for plans without such blocks); psdgb_batch_tuning
 * reads them back, with the number of blocks the on-chip route and of pair
 * tiles the pair shape would take. */
typedef struct psdgb_batch psdgb_batch;
psdgb_status psdgb_batch_create(const int64_t* sizes, int64_t count, int precision, int schedule,
                                psdgb_batch** out);
psdgb_status psdgb_batch_destroy(psdgb_batch* batch);
psdgb_status psdgb_batch_info(const psdgb_batch* batch, int64_t* total_elements, size_t* device_bytes,
                              int64_t* num_tiles, int* acc_mode, int* tile_order);
psdgb_status psdgb_batch_project(psdgb_batch* batch, double* d_blocks, void* stream);
/* The same projection as one CUDA graph launch: the plan captures its
 * kernels once (for this d_blocks pointer and the current configuration; a
 * new pointer, psdgb_batch_configure or psdgb_batch_autotune captures
 * again) and instantiates the graph with the kernels' stream priorities
 * kept, so that the small blocks' high-priority side stream overlaps the
 * larger blocks' work as in psdgb_batch_project (a graph captured by the
 * caller runs every kernel at the priority of the stream it is launched
 * into).  The capture itself must not run inside the caller's own stream
 * capture; later calls only launch the graph on stream. */
psdgb_status psdgb_batch_project_graph(psdgb_batch* batch, double* d_blocks, void* stream);
psdgb_status psdgb_batch_autotune(psdgb_batch* batch, double* d_scratch_blocks, void* stream, double* best_ms);
psdgb_status psdgb_batch_configure(psdgb_batch* batch, int acc_mode, int tile_order, int small_on_chip,
                                   int pair_tiles, int serpentine);
psdgb_status psdgb_batch_tuning(const psdgb_batch* batch, int* acc_mode, int* tile_order, int* small_on_chip,
                                int64_t* small_blocks, int* pair_tiles, int64_t* num_pair_tiles, int* serpentine);

/* ---- eigenpairs and deflation ------------------------------------------------- */
/* Replaces compute_eigenpairs (include/psd_projection/lanczos.h:19-44,
 * src/lanczos.cu:319-547): max_iter Lanczos steps on A (0 = n) with the basis
 * kept, the Ritz pairs of T in order of decreasing |theta|, the residual
 * filter |beta_m Z[0, j]| < ortho_tol (the reference compares with ortho_tol
 * and ignores tol; its residual reads Z's first row) and the orthogonality
 * filter |x_i . x_j| <= ortho_tol against the pairs already taken, up to k
 * pairs.  Unless upper_bound_only, *r_out = r <= k, d_eigenvalues[0..r) and
 * d_eigenvectors (n x r, column-major: vector i at offset i n) are written
 * (k = 0 takes no pair).  *upper_out = |theta_max| + res + 1e-3, the
 * reference's return value.  The start vector is the seeded SplitMix64
 * stream of the Lanczos bound.  Allocates its basis (n (max_iter + 1)
 * doubles) per call, as the reference does; synchronises `stream`. */
psdgb_status psdgb_compute_eigenpairs(const double* d_A, int64_t n, int64_t k, int64_t* r_out, double* d_eigenvalues,
                                      double* d_eigenvectors, int upper_bound_only, int64_t max_iter, double tol,
                                      double ortho_tol, uint64_t seed, double* upper_out, void* stream);
/* Replaces composite_FP32_auto_scale_deflate / composite_FP32_emulated_auto_scale_deflate
 * (include/psd_projection/composite_FP32.h:32-45, src/composite_FP32.cu:193-254,
 * src/composite_FP32_emulated.cu:264-325): the k largest-|lambda| Ritz pairs
 * (psdgb_compute_eigenpairs, max_iter n) are subtracted, the rest is bounded
 * (100 steps, upper_bound_only) and scaled by 1.1 up + 1e-5, filtered with
 * `precision` / `schedule`, scaled back, and the positive pairs are added
 * back.  The second eigenpair run uses seed + 1. */
psdgb_status psdgb_composite_auto_scale_deflate(int precision, int schedule, double* d_mat, int64_t n, int64_t k,
                                                double tol, double ortho_tol, uint64_t seed, void* stream);

/* Replaces lobpcg (include/psd_projection/lobpcg.h, src/lobpcg.cu:12-255):
 * the m largest eigenpairs of the symmetric n x n device matrix A (0 < 3 m <= n)
 * into d_V (n x m, column-major) and d_D (m values, decreasing).  warmstart
 * takes d_V as the (orthonormal) start block, else the seeded stream is
 * orthonormalised; stops when ||A X - X Lambda||_F < tol or after maxiter
 * iterations (*iterations_out).  Synchronises `stream` once per iteration. */
psdgb_status psdgb_lobpcg(const double* d_A, double* d_V, double* d_D, int64_t n, int64_t m, int warmstart,
                          int maxiter, double tol, uint64_t seed, int* iterations_out, void* stream);
/* Replaces eig_FP64_deflate (include/psd_projection/eig_FP64_psd.h:22-31,
 * src/eig_FP64_psd.cu:87-177): the k largest and the k smallest eigenpairs
 * (LOBPCG on X and on -X, maxiter, tol) are subtracted, the rest is projected
 * by the FP64 EVD, and the positive parts are added back.  0 < 3 k <= n. */
psdgb_status psdgb_eig_FP64_deflate(double* d_mat, int64_t n, int64_t k, int maxiter, double tol, uint64_t seed,
                                    void* stream);
/* Replaces composite_FP16_auto_scale_deflate (include/psd_projection/composite_FP16.h:35-50,
 * src/composite_FP16.cu:276-380) for any precision / schedule: the same
 * two-ended deflation, then the Lanczos bound (20 steps), scaling by
 * 1.1 up + 1e-5, the composite filter, scaling back, and the positive parts
 * added back.  0 < 3 k <= n. */
psdgb_status psdgb_composite_auto_scale_deflate_two_ends(int precision, int schedule, double* d_mat, int64_t n,
                                                         int64_t k, int maxiter, double tol, uint64_t seed,
                                                         void* stream);

/* A sequence of `count` n x n host matrices (h_in[i] -> h_out[i]; a buffer
 * may appear more than once and h_out[i] may equal h_in[i], but h_out[i] must
 * not be h_in[i + 1] or h_in[i + 2], which may be read while matrix i is
 * projected or copied back) with one method, pipelined: the host-to-device
 * copies of the next matrices and the device-to-host copy of matrix i - 1 run
 * on their own streams while matrix i is projected on `stream`, through three
 * device staging matrices (an upload waits only for the download three steps
 * earlier).  Copies
 * overlap only for page-locked host buffers (cudaHostAlloc / cudaHostRegister).
 * Returns after the last result is in host memory.  The EVD methods run the
 * matrices one after the other.  No counterpart in the reference, whose
 * MATLAB entry point (MATLAB/psd_projection_MATLAB.cu:93-166) projects one
 * matrix per call. */
psdgb_status psdgb_project_host_many(const char* method, const double* const* h_in, double* const* h_out, int64_t n,
                                     int64_t count, void* stream);

/* ---- diagnostics ------------------------------------------------------------ */
/* Exercises the device-side failure path: one GPU thread waits on an mbarrier
 * that nothing arrives at, with the same bounded-wait code the product
 * kernels use but a limit of limit_seconds (0.001 .. 5); the wait gives up,
 * records a device error word and the kernel returns.  Expected result:
 * PSDGB_ERR_DEVICE_TIMEOUT, with the error word cleared and the context
 * usable afterwards.  No counterpart in the reference. */
psdgb_status psdgb_selftest_wait_timeout(double limit_seconds, void* stream);

/* Accumulator configuration of the tensor-core products of single-matrix
 * calls: -1 = automatic (default: four interleaved K accumulators for long
 * FP32-class products, double-buffered ones otherwise), 0 = four interleaved
 * K accumulators, 1 = two accumulators double-buffered (the epilogue of one
 * tile overlaps the next tile's MMAs), 2 = one accumulator, four buffers.
 * Returns the previous value. */
int psdgb_set_product_config(int acc_mode);
/* Other product-kernel settings, process-wide; returns the previous value
 * (-1 for an unknown knob; out-of-range values are ignored):
 *   PSDGB_TUNE_TILE_GROUP  tile order of single-matrix products: the lower
 *                          tiles are walked in groups of this many tile rows,
 *                          column by column within a group (0 = row by row),
 *                          which sets how many operand row blocks the tiles
 *                          running at the same time share in L2; 0..64;
 *   PSDGB_TUNE_TILE_SHAPE  tile of single-matrix products: -1 = automatic
 *                          (default: 256 x 256 pairs for one- and two-term
 *                          precisions at n > 1920, else 128 x 128); 0 = one
 *                          CTA per 128 x 128 tile; 1 = a CTA pair per
 *                          256 x 128 tile (one tcgen05 MMA over two SMs, each
 *                          supplying half of the B operand); 2 = one CTA per
 *                          128 x 256 tile, K accumulated in chunks summed in
 *                          FP32 registers (one- and two-term precisions; the
 *                          three-term ones keep 128 x 128); 3 = a CTA pair per
 *                          256 x 256 tile (one 256 x 256 x 16 MMA over two
 *                          SMs, K chunks summed in registers, one- and two-term
 *                          precisions);
 *   PSDGB_TUNE_WIDE_KBLOCK K block of a pipeline stage of the 128 x 256 and
 *                          256 x 256 tiles: 0 = by kernel (128 x 256: 32 for
 *                          two-term, 64 for one-term products; 256 x 256: 64),
 *                          64 (128-byte rows) or 32 (64-byte rows, twice the
 *                          stages);
 *   PSDGB_TUNE_GROUP_EPI_WARPS  epilogue warps of the 128 x 128 kernel when it
 *                          runs four accumulator buffers (short K: batches and
 *                          small matrices): 4 or 8;
 *   PSDGB_TUNE_LANCZOS_SYMV  matvec of the Lanczos bound: -1 = automatic
 *                          (default: the lower block triangle in 128 x 128
 *                          tiles from n = 2048), 0 = the whole matrix, a warp
 *                          per column, 1 = the triangle tiles for n >= 128
 *                          (16 consumer warps), 2 = the same with 8. */
enum {
    PSDGB_TUNE_TILE_GROUP = 1,
    PSDGB_TUNE_TILE_SHAPE = 2,
    PSDGB_TUNE_WIDE_KBLOCK = 3,
    PSDGB_TUNE_GROUP_EPI_WARPS = 4,
    PSDGB_TUNE_LANCZOS_SYMV = 5
};
int psdgb_set_product_tuning(int knob, int value);

/* Product-kernel timing: when enabled, the library records a CUDA event pair
 * on the caller's stream around every filter-product launch and adds the
 * elapsed times up when the call synchronises.  psdgb_product_timing_read
 * returns the accumulated milliseconds, launches and executed MMA flops
 * (term products x 2 x 128 x 128 x K per tile) since the last reset. */
psdgb_status psdgb_product_timing_enable(int on);
psdgb_status psdgb_product_timing_read(double* ms, uint64_t* launches, double* mma_flops, int reset);

/* Number of kernels this library launched on the calling process so far. */
uint64_t psdgb_kernel_launch_count(void);
/* Relative Frobenius error ||a - b||_F / ||b||_F of two n x n device FP64
 * matrices, reduced in FP64 on the device. */
psdgb_status psdgb_rel_frobenius(const double* d_a, const double* d_b, int64_t n, double* out,
                                 void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PSDGB_H */
