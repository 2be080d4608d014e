// Classical Gram-Schmidt applied twice (pybte/krylov.py:201-210) for a
// Krylov basis Q[0..j] of long vectors (n ~ 1e5..1e6) and few rows.
//
//   c1 = Q w;  w -= Q^T c1;  c2 = Q w;  w -= Q^T c2;  h = c1 + c2;  h[j+1] = ||w||
//
// Three launches: pass 1 (c1), pass 2 (update by c1, then c2 and h), and the
// last update fused with the norm.  Each launch splits n over kBlocks
// blocks: each thread accumulates all rows over its stride, each warp
// reduces its accumulators with shuffles, and the block's warps are summed in
// warp order into one partial per (block, row).  The last block to finish
// (a fence, then a ticket from an atomic counter -- nothing waits on it) adds
// the block partials per row in block order with a fixed warp tree, so the
// result is deterministic and no separate reduction launch is needed.
//
// Two storage types: FP64 basis (V = double, the FP64 GMRES) and FP32 basis
// (V = float, the inner GMRES of the mixed-precision solve, whose operator
// is an FP32 sweep).  GB300 runs FP64 at 1/64 of the FP32 rate, and the FP64
// products made the FP64 basis the largest cost of an inner Arnoldi column;
// in the FP32 form the products, the per-thread and the warp sums are FP32
// and only the block partials and the cross-block sums are FP64.
#include <cuda_runtime.h>

#include "pbte_internal.cuh"

namespace {

constexpr int kT = 256;
constexpr int kWarps = kT / 32;
constexpr int kBlocks = 304;     // 2 x 152 SMs
constexpr int kMaxRows = 64;

template <typename V>
__device__ __forceinline__ V warp_sum(V v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Scratch layout (doubles): part[kBlocks][kMaxRows], c1[kMaxRows],
// c2[kMaxRows], then the ticket counter (one unsigned, kept at zero between
// calls).
struct Scratch {
    double *part, *c1, *c2;
    unsigned int *ticket;
};

__host__ __device__ inline Scratch scratch_of(double *s) {
    Scratch r;
    r.part = s;
    r.c1 = s + (size_t)kBlocks * kMaxRows;
    r.c2 = r.c1 + kMaxRows;
    r.ticket = reinterpret_cast<unsigned int *>(r.c2 + kMaxRows);
    return r;
}

// Called by every block after it wrote its partials; returns true in the
// one block that arrives last (which then owns the cross-block sums).
__device__ __forceinline__ bool last_block(unsigned int *ticket) {
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (is_last) __threadfence();
    return is_last;
}

// sum over blocks of part[b][k] in a fixed order: warp wid handles rows
// wid, wid + kWarps, ...; lane l adds blocks l, l + 32, ... then the warp
// tree.  Writes out[k] (and out_plus[k] = out[k] + add[k] when given, or the
// square root when `root`).
__device__ void finish_rows(const double *part, int rows, double *out, const double *add, double *out_plus,
                            bool root) {
    const int lane = threadIdx.x % 32, wid = threadIdx.x / 32;
    for (int k = wid; k < rows; k += kWarps) {
        double s = 0.0;
        for (int b = lane; b < kBlocks; b += 32) s += __ldcg(part + (size_t)b * kMaxRows + k);
        s = warp_sum(s);
        if (lane == 0) {
            if (root) {
                out[k] = sqrt(s);
            } else {
                out[k] = s;
                if (out_plus) out_plus[k] = s + add[k];
            }
        }
    }
}

// part[b][k] = sum over this block's entries of Q[k] .* x, where x = w - Q^T c
// when `c` is given (and then w <- x is stored), else x = w.  The last block
// forms out[k] = sum_b part[b][k] (and out_plus = out + add).
template <typename V, int R>
__global__ void __launch_bounds__(kT) multidot_kernel(const V *__restrict__ Q, long long ldq, int rows,
                                                      V *__restrict__ w, const double *__restrict__ c,
                                                      long long n, double *scratch, double *out,
                                                      const double *add, double *out_plus) {
    __shared__ double wsum[kWarps][R];
    const Scratch S = scratch_of(scratch);
    V acc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) acc[k] = V(0);
    V cc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) cc[k] = (c && k < rows) ? (V)c[k] : V(0);
    for (long long t = (long long)blockIdx.x * kT + threadIdx.x; t < n; t += (long long)gridDim.x * kT) {
        V x = w[t];
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
        const V v = warp_sum(acc[k]);
        if (lane == 0) wsum[wid][k] = (double)v;
    }
    __syncthreads();
    if ((int)threadIdx.x < rows) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < kWarps; ++q) s += wsum[q][threadIdx.x];
        S.part[(size_t)blockIdx.x * kMaxRows + threadIdx.x] = s;
    }
    if (last_block(S.ticket)) {
        finish_rows(S.part, rows, out, add, out_plus, false);
        if (threadIdx.x == 0) *S.ticket = 0u;
    }
}

// w -= Q^T c, and the last block forms ||w|| into *norm.
template <typename V, int R>
__global__ void __launch_bounds__(kT) update_norm_kernel(const V *__restrict__ Q, long long ldq, int rows,
                                                         V *__restrict__ w, const double *__restrict__ c,
                                                         long long n, double *scratch, double *norm) {
    __shared__ double wsum[kWarps];
    const Scratch S = scratch_of(scratch);
    V cc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) cc[k] = k < rows ? (V)c[k] : V(0);
    V acc = V(0);
    for (long long t = (long long)blockIdx.x * kT + threadIdx.x; t < n; t += (long long)gridDim.x * kT) {
        V x = w[t];
#pragma unroll
        for (int k = 0; k < R; ++k)
            if (k < rows) x -= Q[k * ldq + t] * cc[k];
        w[t] = x;
        acc += x * x;
    }
    const V v = warp_sum(acc);
    if (threadIdx.x % 32 == 0) wsum[threadIdx.x / 32] = (double)v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < kWarps; ++q) s += wsum[q];
        S.part[(size_t)blockIdx.x * kMaxRows] = s;
    }
    if (last_block(S.ticket)) {
        finish_rows(S.part, 1, norm, nullptr, nullptr, true);
        if (threadIdx.x == 0) *S.ticket = 0u;
    }
}

template <typename V>
int cgs2(const V *Q, int64_t ldq, int32_t rows, V *w, int64_t n, double *h, double *scratch, void *stream) {
    if (!Q || !w || !h || !scratch || rows < 1 || rows > kMaxRows || n < 1 || ldq < n) return PBTE_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const Scratch S = scratch_of(scratch);
    auto go = [&](auto mdot, auto upd) {
        mdot<<<kBlocks, kT, 0, s>>>(Q, ldq, rows, w, nullptr, n, scratch, S.c1, nullptr, nullptr);
        mdot<<<kBlocks, kT, 0, s>>>(Q, ldq, rows, w, S.c1, n, scratch, S.c2, S.c1, h);   // h = c1 + c2
        upd<<<kBlocks, kT, 0, s>>>(Q, ldq, rows, w, S.c2, n, scratch, h + rows);
        return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
    };
    if (rows <= 8) return go(multidot_kernel<V, 8>, update_norm_kernel<V, 8>);
    if (rows <= 16) return go(multidot_kernel<V, 16>, update_norm_kernel<V, 16>);
    if (rows <= 32) return go(multidot_kernel<V, 32>, update_norm_kernel<V, 32>);
    return go(multidot_kernel<V, 64>, update_norm_kernel<V, 64>);
}

}  // namespace

// h[0..rows-1] = c1 + c2 and h[rows] = ||w|| after the two passes; `scratch`
// holds (kBlocks + 3) * 64 doubles, zero before the first call.  rows <= 64.
extern "C" int pbte_cgs2(const double *Q, int64_t ldq, int32_t rows, double *w, int64_t n, double *h,
                         double *scratch, void *stream) {
    return cgs2<double>(Q, ldq, rows, w, n, h, scratch, stream);
}

extern "C" int pbte_cgs2_f32(const float *Q, int64_t ldq, int32_t rows, float *w, int64_t n, double *h,
                             double *scratch, void *stream) {
    return cgs2<float>(Q, ldq, rows, w, n, h, scratch, stream);
}
