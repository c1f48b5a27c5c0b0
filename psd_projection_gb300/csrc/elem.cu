// elem.cu — conversion, operand-split and reduction kernels of the psdgb path.
//
// These replace the reference's per-call conversion and scaling passes
// (convert_double_to_float, convert_float_to_half4 and the Dscal by 1/up,
// src/utils.cu:34-60,106-131, src/composite_FP32.cu:44,184): the FP64 input is
// read once to build the FP32 copy the Lanczos bound streams, and once more to
// write the scaled, split filter operand.  All are HBM-bound.
#include "internal.h"

namespace psdgb {

namespace {

constexpr int TS = 32;  // transpose tile
constexpr int TR = 8;   // rows per thread pass

// Visit the symmetric matrix defined by the upper triangle of the
// column-major x (element (r, c) at x[r + c*n], used where r <= c) one 32x32
// output tile at a time.  The output tile (bi, bj) covers rows i in
// [32 bi, 32 bi + 32) and columns j in [32 bj, 32 bj + 32) of the row-major
// result; the input is read coalesced through a shared-memory transpose.
template <class T, class Store>
__global__ void sym_upper_tiles(const T* __restrict__ x, int64_t n, int64_t rows_out, int64_t cols_out,
                                double scale, const double* scale_dev, Store st) {
    __shared__ double sm[TS][TS + 1];
    if (scale_dev != nullptr) scale *= *scale_dev;
    const int64_t bi = blockIdx.y, bj = blockIdx.x;
    const int tx = threadIdx.x, ty0 = threadIdx.y;
    // Source block: columns (c) of the column-major input are the tile's j
    // when bi <= bj, and its i when bi > bj.
    const int64_t rbase = (bi <= bj) ? bi * TS : bj * TS;  // row range of x read (r)
    const int64_t cbase = (bi <= bj) ? bj * TS : bi * TS;  // column range of x read (c)
    for (int ty = ty0; ty < TS; ty += TR) {
        const int64_t r = rbase + tx, c = cbase + ty;
        sm[ty][tx] = (r < n && c < n) ? static_cast<double>(x[r + c * n]) : 0.0;  // X(rbase+tx, cbase+ty)
    }
    __syncthreads();
    for (int ty = ty0; ty < TS; ty += TR) {
        const int64_t i = bi * TS + ty, j = bj * TS + tx;
        if (i >= rows_out || j >= cols_out) continue;
        double v;
        if (bi < bj) {
            v = sm[tx][ty];                        // X(i, j), i < j
        } else if (bi > bj) {
            v = sm[ty][tx];                        // X(j, i), j < i
        } else {
            v = (ty <= tx) ? sm[tx][ty] : sm[ty][tx];  // diagonal block
        }
        if (i >= n || j >= n) v = 0.0;
        st(i, j, v * scale);
    }
}

struct StoreF32 {
    float* a;
    int64_t ld;
    __device__ void operator()(int64_t i, int64_t j, double v) const { a[i * ld + j] = static_cast<float>(v); }
};

struct StoreSplit {
    SplitMat m;
    int fmt;
    int64_t np;
    __device__ void operator()(int64_t i, int64_t j, double v) const {
        split_store(m, fmt, static_cast<size_t>(i * np + j), static_cast<float>(v));
    }
};

__global__ void split_from_f32_kernel(const float* __restrict__ a, int64_t n, int64_t ld, double scale64,
                                      const double* scale_dev, SplitMat out, int fmt, int64_t np) {
    const float scale = static_cast<float>(scale_dev != nullptr ? scale64 * *scale_dev : scale64);
    const int64_t total = np * np;
    for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < total;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t p = idx / np, q = idx - p * np;
        const float v = (p < n && q < n) ? a[p * ld + q] * scale : 0.0f;
        split_store(out, fmt, static_cast<size_t>(idx), v);
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
    dim3 block(TS, TR), grid(static_cast<unsigned>((ld + TS - 1) / TS), static_cast<unsigned>((n + TS - 1) / TS));
    sym_upper_tiles<double, StoreF32><<<grid, block, 0, s>>>(x, n, n, ld, 1.0, nullptr, StoreF32{a32, ld});
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_sym_upper_f32_to_f32(const float* x, int64_t n, float* a32, int64_t ld, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    dim3 block(TS, TR), grid(static_cast<unsigned>((ld + TS - 1) / TS), static_cast<unsigned>((n + TS - 1) / TS));
    sym_upper_tiles<float, StoreF32><<<grid, block, 0, s>>>(x, n, n, ld, 1.0, nullptr, StoreF32{a32, ld});
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_split_from_f32_upper(const float* x, int64_t n, double scale, const double* scale_dev,
                                        const SplitMat& out, int fmt, int64_t np, cudaStream_t s) {
    dim3 block(TS, TR), grid(static_cast<unsigned>((np + TS - 1) / TS), static_cast<unsigned>((np + TS - 1) / TS));
    sym_upper_tiles<float, StoreSplit><<<grid, block, 0, s>>>(x, n, np, np, scale, scale_dev,
                                                              StoreSplit{out, fmt, np});
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_split_from_f32(const float* a32, int64_t n, int64_t ld, double scale, const double* scale_dev,
                                  const SplitMat& out, int fmt, int64_t np, cudaStream_t s) {
    split_from_f32_kernel<<<grid_for(np * np, 256), 256, 0, s>>>(a32, n, ld, scale, scale_dev, out, fmt, np);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_split_from_f64_upper(const double* x, int64_t n, double scale, const double* scale_dev,
                                        const SplitMat& out, int fmt, int64_t np, cudaStream_t s) {
    dim3 block(TS, TR), grid(static_cast<unsigned>((np + TS - 1) / TS), static_cast<unsigned>((np + TS - 1) / TS));
    sym_upper_tiles<double, StoreSplit><<<grid, block, 0, s>>>(x, n, np, np, scale, scale_dev,
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
