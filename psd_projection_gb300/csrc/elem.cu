// elem.cu — conversion, operand-split and reduction kernels of the psdgb path.
//
// These replace the reference's per-call conversion and scaling passes
// (convert_double_to_float, convert_float_to_half4 and the Dscal by 1/up,
// src/utils.cu:34-60,106-131, src/composite_FP32.cu:44,184): the FP64 input is
// read once to build the FP32 copy the Lanczos bound streams, and once more to
// write the scaled, split filter operand.  All are HBM-bound.
#include "convert.h"
#include "internal.h"

namespace psdgb {

namespace {

constexpr int TS = 32;  // transpose tile
constexpr int TR = 8;   // rows per thread pass

// Visit the symmetric matrix defined by the upper triangle of the
// column-major x (element (r, c) at x[r + c*n], used where r <= c) one pair of
// mirrored 32x32 output tiles at a time: block t reads the source tile of
// rows [32 lo, 32 lo + 32) and columns [32 hi, 32 hi + 32) (lo <= hi) once,
// coalesced, and writes the row-major output tiles (lo, hi) and (hi, lo)
// through a shared-memory transpose (only (lo, lo) on the diagonal).  Each
// upper element is read once: 4 n^2 bytes of FP64 input per matrix.
//
// Values are narrowed to FP32 as they are loaded (FP64 inputs on the integer
// ALUs, convert.h) and scaled in FP32: FP64 instructions issue slowly on this
// GPU and per-element FP64 work made these kernels FP64-bound.  With scale 1
// the stored value is exactly the FP32 rounding of the input.
template <class T>
__device__ __forceinline__ float narrow(T v) { return static_cast<float>(v); }
template <>
__device__ __forceinline__ float narrow<double>(double v) { return d2f_rn(v); }

template <class T, class Store>
__global__ void __launch_bounds__(TS * TR) sym_upper_tiles(const T* __restrict__ x, int64_t n, int64_t rows_out,
                                                           int64_t cols_out, double scale64, const double* scale_dev,
                                                           Store st) {
    __shared__ float sm[TS][TS + 1];
    const float scale = d2f_rn(scale_dev != nullptr ? scale64 * *scale_dev : scale64);
    const bool unscaled = scale == 1.0f;
    // Pair t in row-major order over the tiles (hi, lo), lo <= hi.
    const int64_t t = blockIdx.x;
    // FP32 square root for the estimate (FP64 issues slowly on this GPU); the
    // integer corrections below make it exact.
    int64_t hi = static_cast<int64_t>((sqrtf(8.0f * static_cast<float>(t) + 1.0f) - 1.0f) * 0.5f);
    while (hi * (hi + 1) / 2 > t) --hi;
    while ((hi + 1) * (hi + 2) / 2 <= t) ++hi;
    const int64_t lo = t - hi * (hi + 1) / 2;
    const int tx = threadIdx.x, ty0 = threadIdx.y;
    const int64_t rbase = lo * TS, cbase = hi * TS;
    for (int ty = ty0; ty < TS; ty += TR) {
        const int64_t r = rbase + tx, c = cbase + ty;
        sm[ty][tx] = (r < n && c < n) ? narrow<T>(x[r + c * n]) : 0.0f;  // X(rbase+tx, cbase+ty)
    }
    __syncthreads();
    for (int ty = ty0; ty < TS; ty += TR) {
        {   // tile (lo, hi): X(i, j) with i = rbase + ty <= j = cbase + tx (or the diagonal block)
            const int64_t i = rbase + ty, j = cbase + tx;
            float v = (lo < hi || ty <= tx) ? sm[tx][ty] : sm[ty][tx];
            if (i >= n || j >= n) v = 0.0f;
            if (i < rows_out && j < cols_out) st(i, j, unscaled ? v : v * scale);
        }
        if (lo < hi) {  // tile (hi, lo): X(i, j) = X(j, i), i = cbase + ty, j = rbase + tx
            const int64_t i = cbase + ty, j = rbase + tx;
            float v = sm[ty][tx];
            if (i >= n || j >= n) v = 0.0f;
            if (i < rows_out && j < cols_out) st(i, j, unscaled ? v : v * scale);
        }
    }
}

// Blocks of the pair grid that cover a rows_out x cols_out output.
inline unsigned pair_blocks(int64_t rows_out, int64_t cols_out) {
    const int64_t e = rows_out > cols_out ? rows_out : cols_out;
    const int64_t nt = (e + TS - 1) / TS;
    return static_cast<unsigned>(nt * (nt + 1) / 2);
}

struct StoreF32 {
    float* a;
    int64_t ld;
    __device__ void operator()(int64_t i, int64_t j, float v) const { a[i * ld + j] = v; }
};

struct StoreSplit {
    SplitMat m;
    int fmt;
    int64_t np;
    __device__ void operator()(int64_t i, int64_t j, float v) const {
        split_store(m, fmt, static_cast<size_t>(i * np + j), v);
    }
};

// out = split(a * scale) over the Np x Np operand (zero padding), 8 columns
// per thread: two 16-byte loads (vec: a 16-byte aligned, ld a multiple of 4)
// and one 16-byte store per term plane.
__global__ void split_from_f32_kernel(const float* __restrict__ a, int64_t n, int64_t ld, double scale64,
                                      const double* scale_dev, SplitMat out, int fmt, int64_t np, int vec) {
    const float scale = static_cast<float>(scale_dev != nullptr ? scale64 * *scale_dev : scale64);
    const int64_t chunks = np / 8;
    const int64_t total = np * chunks;
    for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < total;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t p = idx / chunks, q = (idx - p * chunks) * 8;
        float v[8];
        if (vec && p < n && q + 8 <= n) {
            const float4 u0 = *reinterpret_cast<const float4*>(a + p * ld + q);
            const float4 u1 = *reinterpret_cast<const float4*>(a + p * ld + q + 4);
            v[0] = u0.x * scale; v[1] = u0.y * scale; v[2] = u0.z * scale; v[3] = u0.w * scale;
            v[4] = u1.x * scale; v[5] = u1.y * scale; v[6] = u1.z * scale; v[7] = u1.w * scale;
        } else {
#pragma unroll
            for (int e = 0; e < 8; ++e) v[e] = (p < n && q + e < n) ? a[p * ld + q + e] * scale : 0.0f;
        }
        split_store8(out, fmt, static_cast<size_t>(p * np + q), v);
    }
}

__global__ void diff_norms_kernel(const double* __restrict__ a, const double* __restrict__ b, int64_t count,
                                  double* out2) {
    double s_d = 0.0, s_b = 0.0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const double d = a[i] - b[i];
        s_d += d * d;
        s_b += b[i] * b[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        s_d += __shfl_xor_sync(0xffffffffu, s_d, o);
        s_b += __shfl_xor_sync(0xffffffffu, s_b, o);
    }
    __shared__ double red[2][32];
    const int w = threadIdx.x / 32, l = threadIdx.x % 32;
    if (l == 0) { red[0][w] = s_d; red[1][w] = s_b; }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x / 32;
        s_d = (l < nw) ? red[0][l] : 0.0;
        s_b = (l < nw) ? red[1][l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            s_d += __shfl_xor_sync(0xffffffffu, s_d, o);
            s_b += __shfl_xor_sync(0xffffffffu, s_b, o);
        }
        if (l == 0) {
            atomicAdd(out2, s_d);
            atomicAdd(out2 + 1, s_b);
        }
    }
}

template <class T>
__global__ void scale_columns_relu_kernel(T* __restrict__ v, const T* __restrict__ w, int64_t n) {
    const int64_t total = n * n;
    for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < total;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t j = idx / n;
        const T s = w[j] > T(0) ? w[j] : T(0);
        v[idx] *= s;
    }
}

template <class I, class O>
__global__ void convert_kernel(const I* __restrict__ in, O* __restrict__ out, int64_t count) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = static_cast<O>(in[i]);
}

inline unsigned grid_for(int64_t count, int threads) {
    int64_t g = (count + threads - 1) / threads;
    if (g > 152 * 32) g = 152 * 32;
    if (g < 1) g = 1;
    return static_cast<unsigned>(g);
}

}  // namespace

cudaError_t launch_sym_upper_to_f32(const double* x, int64_t n, float* a32, int64_t ld, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const dim3 block(TS, TR);
    sym_upper_tiles<double, StoreF32><<<pair_blocks(n, ld), block, 0, s>>>(x, n, n, ld, 1.0, nullptr,
                                                                           StoreF32{a32, ld});
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_sym_upper_f32_to_f32(const float* x, int64_t n, float* a32, int64_t ld, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const dim3 block(TS, TR);
    sym_upper_tiles<float, StoreF32><<<pair_blocks(n, ld), block, 0, s>>>(x, n, n, ld, 1.0, nullptr,
                                                                          StoreF32{a32, ld});
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_split_from_f32_upper(const float* x, int64_t n, double scale, const double* scale_dev,
                                        const SplitMat& out, int fmt, int64_t np, cudaStream_t s) {
    const dim3 block(TS, TR);
    sym_upper_tiles<float, StoreSplit><<<pair_blocks(np, np), block, 0, s>>>(x, n, np, np, scale, scale_dev,
                                                                             StoreSplit{out, fmt, np});
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_split_from_f32(const float* a32, int64_t n, int64_t ld, double scale, const double* scale_dev,
                                  const SplitMat& out, int fmt, int64_t np, cudaStream_t s) {
    const int vec = (reinterpret_cast<uintptr_t>(a32) & 15u) == 0 && ld % 4 == 0;
    split_from_f32_kernel<<<grid_for(np * np / 8, 256), 256, 0, s>>>(a32, n, ld, scale, scale_dev, out, fmt, np,
                                                                      vec);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_split_from_f64_upper(const double* x, int64_t n, double scale, const double* scale_dev,
                                        const SplitMat& out, int fmt, int64_t np, cudaStream_t s) {
    const dim3 block(TS, TR);
    sym_upper_tiles<double, StoreSplit><<<pair_blocks(np, np), block, 0, s>>>(x, n, np, np, scale, scale_dev,
                                                                              StoreSplit{out, fmt, np});
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_diff_norms(const double* a, const double* b, int64_t count, double* d_out2, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(d_out2, 0, 2 * sizeof(double), s);
    if (e != cudaSuccess) return e;
    if (count == 0) return cudaSuccess;
    diff_norms_kernel<<<grid_for(count, 256), 256, 0, s>>>(a, b, count, d_out2);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_scale_columns_relu(double* v, const double* w, int64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    scale_columns_relu_kernel<double><<<grid_for(n * n, 256), 256, 0, s>>>(v, w, n);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_scale_columns_relu_f32(float* v, const float* w, int64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    scale_columns_relu_kernel<float><<<grid_for(n * n, 256), 256, 0, s>>>(v, w, n);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_f64_to_f32(const double* in, float* out, int64_t count, cudaStream_t s) {
    if (count == 0) return cudaSuccess;
    convert_kernel<double, float><<<grid_for(count, 256), 256, 0, s>>>(in, out, count);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_f32_to_f64(const float* in, double* out, int64_t count, cudaStream_t s) {
    if (count == 0) return cudaSuccess;
    convert_kernel<float, double><<<grid_for(count, 256), 256, 0, s>>>(in, out, count);
    count_launch();
    return cudaGetLastError();
}

// Self-test of the bounded waits: one thread waits on an mbarrier that no
// thread or copy ever arrives at; the wait gives up after limit_ns and records
// DEVERR_SELFTEST_WAIT, and the kernel returns with nothing in flight.
__global__ void wait_selftest_kernel(int* err, uint64_t limit_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0 && !mbar_wait_limit(&bar, 0, limit_ns)) atomicCAS(err, 0, DEVERR_SELFTEST_WAIT);
}

cudaError_t launch_wait_selftest(int* err, uint64_t limit_ns, cudaStream_t s) {
    wait_selftest_kernel<<<1, 32, 0, s>>>(err, limit_ns);
    count_launch();
    return cudaGetLastError();
}

}  // namespace psdgb
