// Classical Gram-Schmidt applied twice (pybte/krylov.py:201-210), FP64, for
// a Krylov basis Q[0..j] of long vectors (n ~ 1e5..1e6) and few rows.
//
//   c1 = Q w;  w -= Q^T c1;  c2 = Q w;  w -= Q^T c2;  h = c1 + c2;  h[j+1] = ||w||
//
// The row-dot products split n over kBlocks blocks: each thread accumulates
// all rows over its stride, each warp reduces its accumulators with
// shuffles, and the block's warps are summed in warp order into one partial
// per (block, row).  A second kernel adds the block partials per row with a
// fixed-shape tree, so the result is deterministic.  The update of w is
// fused with the next product, and the last update with the norm.
#include <cuda_runtime.h>

#include "pbte_internal.cuh"

namespace {

constexpr int kT = 256;
constexpr int kWarps = kT / 32;
constexpr int kBlocks = 304;     // 2 x 152 SMs
constexpr int kMaxRows = 64;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// part[b][k] = sum over this block's entries of Q[k] .* x, where x = w - Q^T c
// when `c` is given (and then w <- x is stored), else x = w.
template <int R>
__global__ void __launch_bounds__(kT) multidot_kernel(const double *__restrict__ Q, long long ldq, int rows,
                                                      double *__restrict__ w, const double *__restrict__ c,
                                                      long long n, double *__restrict__ part) {
    __shared__ double wsum[kWarps][R];
    double acc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) acc[k] = 0.0;
    double cc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) cc[k] = (c && k < rows) ? c[k] : 0.0;
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
    const int lane = threadIdx.x % 32, wid = threadIdx.x / 32;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const double v = warp_sum(acc[k]);
        if (lane == 0) wsum[wid][k] = v;
    }
    __syncthreads();
    if ((int)threadIdx.x < rows) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < kWarps; ++q) s += wsum[q][threadIdx.x];
        part[(size_t)blockIdx.x * kMaxRows + threadIdx.x] = s;
    }
}

// One block per row: out[k] = sum_b part[b][k] (+ add[k]) by a fixed tree.
__global__ void __launch_bounds__(kT) sum_parts_kernel(const double *part, int rows, const double *add, double *out,
                                                       int sqrt_out) {
    __shared__ double red[kT];
    const int k = blockIdx.x;
    double s = 0.0;
    for (int b = threadIdx.x; b < kBlocks; b += kT) s += part[(size_t)b * kMaxRows + k];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = kT / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double v = red[0] + (add ? add[k] : 0.0);
        out[k] = sqrt_out ? sqrt(v) : v;
    }
    (void)rows;
}

// w -= Q^T c and the block partials of ||w||^2 (row 0 of part).
template <int R>
__global__ void __launch_bounds__(kT) update_norm_kernel(const double *__restrict__ Q, long long ldq, int rows,
                                                         double *__restrict__ w, const double *__restrict__ c,
                                                         long long n, double *__restrict__ part) {
    __shared__ double wsum[kWarps];
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
    const double v = warp_sum(acc);
    if (threadIdx.x % 32 == 0) wsum[threadIdx.x / 32] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < kWarps; ++q) s += wsum[q];
        part[(size_t)blockIdx.x * kMaxRows] = s;
    }
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
        sum_parts_kernel<<<rows, kT, 0, s>>>(part, rows, nullptr, c1, 0);
        mdot<<<kBlocks, kT, 0, s>>>(Q, ldq, rows, w, c1, n, part);
        sum_parts_kernel<<<rows, kT, 0, s>>>(part, rows, c1, h, 0);     // h = c1 + c2 ...
        sum_parts_kernel<<<rows, kT, 0, s>>>(part, rows, nullptr, c2, 0);
        upd<<<kBlocks, kT, 0, s>>>(Q, ldq, rows, w, c2, n, part);
        sum_parts_kernel<<<1, kT, 0, s>>>(part, 1, nullptr, h + rows, 1);
        return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
    };
    if (rows <= 8) return go(multidot_kernel<8>, update_norm_kernel<8>);
    if (rows <= 16) return go(multidot_kernel<16>, update_norm_kernel<16>);
    if (rows <= 32) return go(multidot_kernel<32>, update_norm_kernel<32>);
    return go(multidot_kernel<64>, update_norm_kernel<64>);
}
