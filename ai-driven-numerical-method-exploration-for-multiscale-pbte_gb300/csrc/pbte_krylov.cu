// Classical Gram-Schmidt applied twice (pybte/krylov.py:201-210), FP64, for
// a Krylov basis Q[0..j] of long vectors (n ~ 1e5..1e6) and few rows.
//
//   c1 = Q w;  w -= Q^T c1;  c2 = Q w;  w -= Q^T c2;  h = c1 + c2;  h[j+1] = ||w||
//
// The row-dot products split n over many blocks (each thread accumulates all
// j+1 rows over its stride, a block tree-reduces them into one partial per
// row) and a second pass adds the block partials in block order, so the
// result is deterministic.  The update of w is fused with the next product.
#include <cuda_runtime.h>

#include "pbte_internal.cuh"

namespace {

constexpr int kT = 256;
constexpr int kBlocks = 608;     // 4 x 152 SMs
constexpr int kMaxRows = 64;

// part[b][k] = sum over this block's entries of Q[k] .* x, where x = w - Q^T c
// when `c` is given (and then w <- x is stored), else x = w.
template <int R>
__global__ void __launch_bounds__(kT) multidot_kernel(const double *__restrict__ Q, long long ldq, int rows,
                                                      double *__restrict__ w, const double *__restrict__ c,
                                                      long long n, double *__restrict__ part) {
    __shared__ double red[kT];
    double acc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) acc[k] = 0.0;
    double cc[R];
    if (c) {
#pragma unroll
        for (int k = 0; k < R; ++k) cc[k] = k < rows ? c[k] : 0.0;
    }
    for (long long t = (long long)blockIdx.x * kT + threadIdx.x; t < n; t += (long long)gridDim.x * kT) {
        double x = w[t];
        if (c) {
#pragma unroll
            for (int k = 0; k < R; ++k)
                if (k < rows) x -= Q[k * ldq + t] * cc[k];
            w[t] = x;
        }
#pragma unroll
        for (int k = 0; k < R; ++k)
            if (k < rows) acc[k] += Q[k * ldq + t] * x;
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (k >= rows) break;
        red[threadIdx.x] = acc[k];
        __syncthreads();
        for (int h = kT / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
            __syncthreads();
        }
        if (threadIdx.x == 0) part[(size_t)blockIdx.x * kMaxRows + k] = red[0];
        __syncthreads();
    }
}

// out[k] = sum_b part[b][k] (block order), plus add_to[k] when given.
__global__ void sum_parts_kernel(const double *part, int nblocks, int rows, const double *add, double *out) {
    const int k = threadIdx.x;
    if (k >= rows) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += part[(size_t)b * kMaxRows + k];
    out[k] = add ? s + add[k] : s;
}

// w -= Q^T c and the block partials of ||w||^2.
template <int R>
__global__ void __launch_bounds__(kT) update_norm_kernel(const double *__restrict__ Q, long long ldq, int rows,
                                                         double *__restrict__ w, const double *__restrict__ c,
                                                         long long n, double *__restrict__ part) {
    __shared__ double red[kT];
    double cc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) cc[k] = k < rows ? c[k] : 0.0;
    double acc = 0.0;
    for (long long t = (long long)blockIdx.x * kT + threadIdx.x; t < n; t += (long long)gridDim.x * kT) {
        double x = w[t];
#pragma unroll
        for (int k = 0; k < R; ++k)
            if (k < rows) x -= Q[k * ldq + t] * cc[k];
        w[t] = x;
        acc += x * x;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int h = kT / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[(size_t)blockIdx.x * kMaxRows] = red[0];
}

__global__ void sqrt_sum_kernel(const double *part, int nblocks, double *out) {
    if (threadIdx.x != 0) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += part[(size_t)b * kMaxRows];
    *out = sqrt(s);
}

__global__ void add_vec_kernel(const double *a, const double *b, int rows, double *out) {
    const int k = threadIdx.x;
    if (k < rows) out[k] = a[k] + b[k];
}

}  // namespace

// h[0..rows-1] = c1 + c2 and h[rows] = ||w|| after the two passes; `scratch`
// holds (kBlocks + 2) * 64 doubles.  rows <= 64.
extern "C" int pbte_cgs2(const double *Q, int64_t ldq, int32_t rows, double *w, int64_t n, double *h,
                         double *scratch, void *stream) {
    if (!Q || !w || !h || !scratch || rows < 1 || rows > kMaxRows || n < 1 || ldq < n) return PBTE_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    double *part = scratch;
    double *c1 = scratch + (size_t)kBlocks * kMaxRows;
    double *c2 = c1 + kMaxRows;
    auto go = [&](auto mdot, auto upd) {
        mdot<<<kBlocks, kT, 0, s>>>(Q, ldq, rows, w, nullptr, n, part);
        sum_parts_kernel<<<1, kMaxRows, 0, s>>>(part, kBlocks, rows, nullptr, c1);
        mdot<<<kBlocks, kT, 0, s>>>(Q, ldq, rows, w, c1, n, part);
        sum_parts_kernel<<<1, kMaxRows, 0, s>>>(part, kBlocks, rows, nullptr, c2);
        upd<<<kBlocks, kT, 0, s>>>(Q, ldq, rows, w, c2, n, part);
        add_vec_kernel<<<1, kMaxRows, 0, s>>>(c1, c2, rows, h);
        sqrt_sum_kernel<<<1, 32, 0, s>>>(part, kBlocks, h + rows);
        return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
    };
    if (rows <= 8) return go(multidot_kernel<8>, update_norm_kernel<8>);
    if (rows <= 16) return go(multidot_kernel<16>, update_norm_kernel<16>);
    if (rows <= 32) return go(multidot_kernel<32>, update_norm_kernel<32>);
    return go(multidot_kernel<64>, update_norm_kernel<64>);
}
