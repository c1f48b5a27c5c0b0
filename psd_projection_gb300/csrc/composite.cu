// composite.cu — host orchestration of the composite polynomial filter.
//
// Restates the control flow of composite_FP32 / composite_FP16 /
// composite_FP32_emulated (src/composite_FP32.cu:15-164,
// src/composite_FP16.cu:16-246, src/composite_FP32_emulated.cu:20-235) and
// their _auto_scale wrappers (src/composite_FP32.cu:166-191 and the FP16 /
// emulated twins), on the fused kernels of this library:
//
//   prologue  FP64 input -> FP32 copy for the Lanczos bound -> scaled operand
//             terms (padded to a multiple of 128, zero padding);
//   per step  A2 = A*A; A3 = A2*A; A = a*A + b*A3 + c*A3*A2   (three products,
//             the coefficient combination fused into the third epilogue);
//   final     out = (X + up * (Xs*A + A*Xs)/2) / 2 with Xs = X / up, fused into
//             the last product's epilogue, written in FP64 in place — the same
//             matrix as the reference's sym(Xs * (I + A) / 2) times up
//             (:142-156, :190).  The symmetric part is one K-concatenated
//             product on one triangle: [Xs | A] * [A | Xs]^T.
//
// Workspace: three split matrices (A, A2, A3) of Np x Np, Np = n rounded up
// to 128.  The FP32 copy the Lanczos bound streams lives in A2's storage
// (A2 is not in use until the first product), and the final product's Xs
// operand is written into A2's storage as well.
#include <cmath>
#include <vector>

#include "internal.h"

namespace psdgb {

namespace {

// Quintic coefficients (a, b, c) of the sign filter, src/composite_FP32.cu:73-84
// ("polar express refined", 10 steps; also src/composite_FP32_emulated.cu:78-89).
const double kCoeffFP32[10][3] = {
    {8.3119043343, -23.0739115930, 16.4664144722}, {4.1439360087, -2.9176674704, 0.5246212487},
    {4.0257813209, -2.9025002398, 0.5334261214},   {3.5118574347, -2.5740236523, 0.5050097282},
    {2.4398158400, -1.7586675341, 0.4191290613},   {1.9779835097, -1.3337358510, 0.3772169049},
    {1.9559726949, -1.3091355170, 0.3746734515},   {1.9282822454, -1.2823649693, 0.3704626545},
    {1.9220135179, -1.2812524618, 0.3707011753},   {1.8942192942, -1.2613293407, 0.3676616051}};
// src/composite_FP16.cu:93-101 ("polar express with refinement", 7 steps).
const double kCoeffFP16[7][3] = {
    {8.2885332412, -22.5927099246, 15.8201383114}, {4.1666196466, -2.9679004036, 0.5307623217},
    {4.0611848147, -2.9698947955, 0.5492133813},   {3.6678301399, -2.7561018955, 0.5421513305},
    {2.7632556383, -2.0607754898, 0.4695405857},   {2.0527445797, -1.4345145882, 0.4070669182},
    {1.8804816691, -1.2583997294, 0.3779501813}};

}  // namespace

struct Step {
    float a, b, c;
};

// The per-step coefficients after the safety scaling p(x / s), computed in
// FP32 exactly as the reference does (src/composite_FP32.cu:86-99: s = 1.001
// on steps 0-7; src/composite_FP16.cu:103-113: s = 1.01 on every step).
std::vector<Step> schedule_steps(int schedule) {
    std::vector<Step> out;
    if (schedule == PSDGB_SCHEDULE_FP16 || schedule == PSDGB_SCHEDULE_FP8) {
        const float s = schedule == PSDGB_SCHEDULE_FP8 ? 1.5f : 1.01f;
        for (auto& r : kCoeffFP16) {
            float a = static_cast<float>(r[0]), b = static_cast<float>(r[1]), c = static_cast<float>(r[2]);
            a /= s;
            b /= s * s * s;
            c /= s * s * s * s * s;
            out.push_back({a, b, c});
        }
    } else {
        const float s = 1.001f;
        for (int i = 0; i < 10; ++i) {
            float a = static_cast<float>(kCoeffFP32[i][0]), b = static_cast<float>(kCoeffFP32[i][1]),
                  c = static_cast<float>(kCoeffFP32[i][2]);
            if (i < 8) {
                a /= s;
                b /= s * s * s;
                c /= s * s * s * s * s;
            }
            out.push_back({a, b, c});
        }
    }
    return out;
}

namespace {

struct Layout {
    int fmt;
    int64_t np;
    size_t mat_bytes;
    SplitMat A, A2, A3;
    float* a32;   // FP32 copy of the input (n x ld), inside A2's storage
    int64_t ld;   // = n rounded up to 4
};

Layout make_layout(void* ws, int fmt, int64_t n) {
    Layout L{};
    L.fmt = fmt;
    L.np = pad128(n);
    const size_t elems = static_cast<size_t>(L.np) * L.np;
    const int nt = format_terms(fmt);
    L.mat_bytes = elems * format_bytes(fmt);
    char* base = static_cast<char*>(ws);
    SplitMat* mats[3] = {&L.A, &L.A2, &L.A3};
    for (int m = 0; m < 3; ++m) {
        size_t off = m * L.mat_bytes;
        for (int t = 0; t < 3; ++t) {
            mats[m]->term[t] = (t < nt) ? base + off : nullptr;
            if (t < nt) off += elems * format_plane_bytes(fmt, t);
        }
    }
    L.a32 = reinterpret_cast<float*>(L.A2.term[0]);
    L.ld = (n + 3) / 4 * 4;
    return L;
}

// Epilogue parameters of a product at `precision` on layout L.  Only E4M3
// products read the F16Q8 format's E4M3 plane; the FP16 products that refine
// an FP8 bulk read and write the FP16 pair alone (planes 0 and 1, laid out as
// the F16 format), so their epilogues store the F16 format.
EpiParams epi_base(const Layout& L, int64_t n, int precision) {
    EpiParams ep{};
    ep.fmt = (L.fmt == FMT_F16Q8 && precision != PSDGB_PREC_FP8) ? FMT_F16 : L.fmt;
    ep.np = static_cast<int>(L.np);
    ep.n = static_cast<int>(n);
    ep.acc_scale = 1.0f;
    ep.ld = static_cast<int>(L.np);
    return ep;
}

// One filter step A <- a A + b A^3 + c A^5 (three products) at a precision.
psdgb_status run_step(DeviceState* ds, int precision, const Step& st, const Layout& L, int64_t n, cudaStream_t s) {
    PrecisionInfo pi{};
    precision_info(precision, &pi);
    // One-term operands round to 11 (FP16) or 8 (BF16) bits; the antisymmetric
    // part of that rounding error in A2*A and A3*A2 is pure error, so those
    // modes take the symmetric parts (A2*A + A*A2)/2 and (A3*A2 + A2*A3)/2 as
    // dual products, as the reference symmetrises A after every step
    // (src/composite_FP16.cu:166).  (Measured on the CPU model at n = 300 to
    // 1200: relative error 1.12-1.16x the reference FP16 method's with the
    // third product dual alone, 1.02-1.03x with both.)
    const bool dual_step = pi.nprod == 1;
    {
        EpiParams e1 = epi_base(L, n, precision);
        e1.kind = EPI_STORE;
        e1.out = L.A2;
        PSDGB_TRY(gemm_symmetric(ds, precision, L.A, L.A, L.np, e1, s));  // A2 = A * A
        EpiParams e2 = epi_base(L, n, precision);
        e2.kind = EPI_STORE;
        e2.out = L.A3;
        if (dual_step) {
            e2.dual = 1;
            e2.acc_scale = 0.5f;
        }
        PSDGB_TRY(gemm_symmetric(ds, precision, L.A2, L.A, L.np, e2, s));  // A3 = A2 * A
        EpiParams e3 = epi_base(L, n, precision);
        e3.kind = EPI_STEP;
        e3.a = st.a;
        e3.b = st.b;
        e3.c = st.c;
        e3.A = L.A;
        e3.A3 = L.A3;
        e3.out = L.A;
        if (dual_step) {
            e3.dual = 1;
            e3.acc_scale = 0.5f;
        }
        PSDGB_TRY(gemm_symmetric(ds, precision, L.A3, L.A2, L.np, e3, s));  // A = aA + bA3 + cA3*A2
    }
    return PSDGB_OK;
}

// The whole schedule at one precision; or, with bulk_precision >= 0, the
// schedule at bulk_precision followed by refine_steps steps of the
// Newton-Schulz-type quintic that ends the FP32 table (no safety factor) at
// `precision` — a low-precision bulk with higher-precision refinement.
psdgb_status run_filter(DeviceState* ds, int precision, int schedule, const Layout& L, int64_t n, cudaStream_t s,
                        int bulk_precision = -1, int refine_steps = 0) {
    const int bulk = bulk_precision >= 0 ? bulk_precision : precision;
    for (const Step& st : schedule_steps(schedule)) PSDGB_TRY(run_step(ds, bulk, st, L, n, s));
    if (bulk_precision >= 0) {
        const Step fin = schedule_steps(PSDGB_SCHEDULE_FP32).back();
        for (int r = 0; r < refine_steps; ++r) PSDGB_TRY(run_step(ds, precision, fin, L, n, s));
    }
    return PSDGB_OK;
}

// mat (in place) = (X + up * (Xs*A + A*Xs)/2) / 2, Xs = X / up, X read from
// mat; up is up_host times the device value up_dev when given.
psdgb_status run_final(DeviceState* ds, int precision, const Layout& L, double* mat, int64_t n, const double* up_dev,
                       const double* inv_up_dev, cudaStream_t s, double up_host = 1.0) {
    PSDGB_CUDA_TRY(launch_split_from_f64_upper(mat, n, 1.0 / up_host, inv_up_dev, L.A2, L.fmt, L.np, s));
    EpiParams ef = epi_base(L, n, precision);
    ef.kind = EPI_FINAL;
    ef.up = up_host;
    ef.up_dev = up_dev;
    // (Xs*A + A*Xs)/2: the symmetric part of the product, as the reference's
    // symmetrisation of W does (src/composite_FP32.cu:153).
    ef.dual = 1;
    ef.acc_scale = 0.5f;
    ef.x64 = mat;
    ef.out64 = mat;
    return gemm_symmetric(ds, precision, L.A2, L.A, L.np, ef, s);
}

psdgb_status check_n(int64_t n) {
    if (n < 0) {
        set_error("matrix size must be >= 0");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (n > 46340 * 2) {  // Np^2 indices and tile counts stay in range
        set_error("matrix size too large (n <= 92680)");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    return PSDGB_OK;
}

}  // namespace

bool precision_info(int precision, PrecisionInfo* out) {
    switch (precision) {
        case PSDGB_PREC_FP32_SIMT: *out = {FMT_F32, 0, 1}; return true;
        case PSDGB_PREC_FP16: *out = {FMT_F16, 1, 1}; return true;
        case PSDGB_PREC_BF16: *out = {FMT_BF16, 1, 1}; return true;
        case PSDGB_PREC_FP16X3: *out = {FMT_F16, 3, 2}; return true;
        case PSDGB_PREC_BF16X3: *out = {FMT_BF16, 3, 2}; return true;
        case PSDGB_PREC_BF16X6: *out = {FMT_BF16, 6, 3}; return true;
        case PSDGB_PREC_BF16X9: *out = {FMT_BF16, 9, 3}; return true;
        case PSDGB_PREC_FP8: *out = {FMT_F16Q8, 1, 1}; return true;
        default: return false;
    }
}

size_t split_matrix_bytes(int fmt, int64_t np) {
    return static_cast<size_t>(np) * np * format_bytes(fmt);
}

psdgb_status gemm_symmetric(DeviceState* ds, int precision, const SplitMat& P, const SplitMat& Q, int64_t np,
                            const EpiParams& ep, cudaStream_t s) {
    PrecisionInfo pi{};
    precision_info(precision, &pi);
    const double nt = static_cast<double>(np / 128);
    const double flops = nt * (nt + 1) / 2 * 2.0 * 128 * 128 * static_cast<double>(np) * (ep.dual ? 2 : 1) *
                         (pi.nprod > 0 ? pi.nprod : 1);
    product_timing_begin(s);
    psdgb_status st = (precision == PSDGB_PREC_FP32_SIMT) ? gemm_simt(ds, P, Q, np, ep, s)
                                                           : gemm_tc(ds, precision, P, Q, np, ep, s);
    product_timing_end(s, flops);
    return st;
}

size_t composite_ws_bytes(int64_t n, int precision) {
    PrecisionInfo pi{};
    if (!precision_info(precision, &pi) || n <= 0) return 0;
    return 3 * split_matrix_bytes(pi.fmt, pad128(n));
}

psdgb_status composite_enqueue(DeviceState* ds, int precision, int schedule, double* mat, int64_t n, void* ws,
                               bool auto_scale, int64_t max_iter, double tol, uint64_t seed, int residual_mode,
                               void* lz_state, cudaStream_t s, const double* d_warm, double* d_ritz_out,
                               int bulk_precision, int refine_steps) {
    PSDGB_TRY(check_n(n));
    PrecisionInfo pi{};
    if (!precision_info(precision, &pi)) {
        set_error("unknown precision");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (const char* why = schedule_error(bulk_precision >= 0 ? bulk_precision : precision, schedule)) {
        set_error(why);
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return PSDGB_OK;
    // An FP8 bulk stores its operands in the F16Q8 format (the E4M3 plane for
    // its products beside the FP16 pair the refinement reads).
    const Layout L = make_layout(ws, bulk_precision == PSDGB_PREC_FP8 ? FMT_F16Q8 : pi.fmt, n);
    const double* up_dev = nullptr;
    const double* inv_up_dev = nullptr;
    if (auto_scale) {
        // The bound runs on the device and leaves scale = up > 0 ? up : 1
        // (src/composite_FP32.cu:182) and its inverse in the Lanczos state,
        // which the split kernels and the final epilogue read: no host round trip.
        PSDGB_CUDA_TRY(launch_sym_upper_to_f32(mat, n, L.a32, L.ld, s));
        PSDGB_TRY(lanczos_bound_async(ds, L.a32, n, L.ld, max_iter, tol, seed, residual_mode, lz_state, s, d_warm,
                                      d_ritz_out));
        up_dev = lanczos_scale_ptr(lz_state, n, max_iter);
        inv_up_dev = lanczos_inv_scale_ptr(lz_state, n, max_iter);
        PSDGB_CUDA_TRY(launch_split_from_f32(L.a32, n, L.ld, 1.0, inv_up_dev, L.A, L.fmt, L.np, s));
    } else {
        PSDGB_CUDA_TRY(launch_split_from_f64_upper(mat, n, 1.0, nullptr, L.A, L.fmt, L.np, s));
    }
    PSDGB_TRY(run_filter(ds, precision, schedule, L, n, s, bulk_precision, refine_steps));
    PSDGB_TRY(run_final(ds, precision, L, mat, n, up_dev, inv_up_dev, s));
    return PSDGB_OK;
}

// The filter of a matrix scaled by 1 / scale (a host value), and its result
// scaled back: the reference's Dscal(1/scale), composite, Dscal(scale)
// (src/composite_FP32.cu:233-243), with both scalings folded into the first
// operand split and the final epilogue.
psdgb_status composite_enqueue_scaled(DeviceState* ds, int precision, int schedule, double* mat, int64_t n, void* ws,
                                      double scale, cudaStream_t s) {
    PSDGB_TRY(check_n(n));
    PrecisionInfo pi{};
    if (!precision_info(precision, &pi)) {
        set_error("unknown precision");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return PSDGB_OK;
    if (!(scale > 0.0)) scale = 1.0;
    const Layout L = make_layout(ws, pi.fmt, n);
    PSDGB_CUDA_TRY(launch_split_from_f64_upper(mat, n, 1.0 / scale, nullptr, L.A, L.fmt, L.np, s));
    PSDGB_TRY(run_filter(ds, precision, schedule, L, n, s, -1, 0));
    return run_final(ds, precision, L, mat, n, nullptr, nullptr, s, scale);
}

// The auto-scaled projection of a column-major FP32 matrix, in place (its
// upper triangle defines it): the FP32 copy for the bound comes from the FP32
// input, the final operand split reads it, and the final epilogue writes
// FP32 (its arithmetic in FP64).  Asynchronous, like composite_enqueue.
psdgb_status composite_enqueue_f32(DeviceState* ds, int precision, int schedule, float* mat, int64_t n, void* ws,
                                   int64_t max_iter, double tol, uint64_t seed, int residual_mode, void* lz_state,
                                   cudaStream_t s, const double* d_warm, double* d_ritz_out) {
    PSDGB_TRY(check_n(n));
    PrecisionInfo pi{};
    if (!precision_info(precision, &pi) || precision == PSDGB_PREC_FP32_SIMT) {
        set_error("FP32 input needs a tensor-core precision");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (const char* why = schedule_error(precision, schedule)) {
        set_error(why);
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return PSDGB_OK;
    const Layout L = make_layout(ws, pi.fmt, n);
    PSDGB_CUDA_TRY(launch_sym_upper_f32_to_f32(mat, n, L.a32, L.ld, s));
    PSDGB_TRY(lanczos_bound_async(ds, L.a32, n, L.ld, max_iter, tol, seed, residual_mode, lz_state, s, d_warm,
                                  d_ritz_out));
    const double* up_dev = lanczos_scale_ptr(lz_state, n, max_iter);
    const double* inv_up_dev = lanczos_inv_scale_ptr(lz_state, n, max_iter);
    PSDGB_CUDA_TRY(launch_split_from_f32(L.a32, n, L.ld, 1.0, inv_up_dev, L.A, L.fmt, L.np, s));
    PSDGB_TRY(run_filter(ds, precision, schedule, L, n, s, -1, 0));
    PSDGB_CUDA_TRY(launch_split_from_f32_upper(mat, n, 1.0, inv_up_dev, L.A2, L.fmt, L.np, s));
    EpiParams ef = epi_base(L, n, precision);
    ef.kind = EPI_FINAL32;
    ef.up = 1.0;
    ef.up_dev = up_dev;
    ef.dual = 1;
    ef.acc_scale = 0.5f;
    ef.x32 = mat;
    ef.out32 = mat;
    return gemm_symmetric(ds, precision, L.A2, L.A, L.np, ef, s);
}

psdgb_status composite_run(DeviceState* ds, int precision, int schedule, double* mat, int64_t n, void* ws,
                           bool auto_scale, int64_t max_iter, double tol, uint64_t seed, int residual_mode,
                           void* lz_state, cudaStream_t s, double* up_out) {
    if (up_out) *up_out = 1.0;
    PSDGB_TRY(composite_enqueue(ds, precision, schedule, mat, n, ws, auto_scale, max_iter, tol, seed, residual_mode,
                                lz_state, s, nullptr, nullptr, -1, 0));
    if (up_out && auto_scale && n > 0) {
        LanczosResult lr;
        PSDGB_TRY(lanczos_read(lz_state, n, max_iter, s, &lr, nullptr, nullptr));
        *up_out = lr.up > 0.0 ? lr.up : 1.0;
    }
    return PSDGB_OK;
}

}  // namespace psdgb

extern "C" int psdgb_filter_coefficients(int schedule, float* out, int cap) {
    if (schedule != PSDGB_SCHEDULE_FP32 && schedule != PSDGB_SCHEDULE_FP16 && schedule != PSDGB_SCHEDULE_FP8) return -1;
    const std::vector<psdgb::Step> steps = psdgb::schedule_steps(schedule);
    for (int i = 0; i < cap && i < static_cast<int>(steps.size()); ++i) {
        out[3 * i] = steps[i].a;
        out[3 * i + 1] = steps[i].b;
        out[3 * i + 2] = steps[i].c;
    }
    return static_cast<int>(steps.size());
}
