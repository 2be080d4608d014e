// Device solve of the GSIS trace system with a nested-dissection
// multifrontal factorisation (factors built on the host by
// pbte_gb300/trace_nd.py; replaces the SuperLU triangular solves of
// pybte/acceleration/global_solve.py:189-195).
//
// Per tree node (front) the host stores
//   G = [L11^-1 P ; -L21 L11^-1 P]   (m x o, row-major)
//   H = [U11^-1, -U11^-1 U12]        (o x m, row-major)
// for its o own and m - o boundary unknowns.  The forward sweep runs the
// nodes by height (leaves first): the node's own right-hand side is the
// original one plus its children's boundary updates, y = G_top v goes to z,
// and its own boundary update G_bot v plus the children's updates to those
// unknowns goes to its delta slots.  The backward sweep (root first) forms
// x_own = H [z_own ; x_bnd].  One thread block per work item (a node and a
// run of output rows, laid out by the host); a warp per row, lanes striding
// the columns (coalesced, four loads in flight per lane), the input vector in
// shared memory.  Sums are in a fixed order, so the solve is deterministic.
#include <cuda_runtime.h>

#include "pbte_internal.cuh"

namespace {

constexpr int kThreads = 256;

// node metadata, int64 each: index offset, own count o, front size m,
// G offset, H offset, delta offset, contribution-pointer offset, pad
struct NodeMeta {
    int64_t ioff, o, m, goff, hoff, doff, coff, pad;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
    return v;
}

__device__ __forceinline__ double gather_updates(const int64_t *cptr, const int64_t *csrc, const double *delta,
                                                 int64_t at) {
    double s = 0.0;
    for (int64_t e = cptr[at]; e < cptr[at + 1]; ++e) s += delta[csrc[e]];
    return s;
}

__global__ void __launch_bounds__(kThreads) nd_forward_kernel(const int4 *items, const NodeMeta *meta,
                                                              const int32_t *idx, const int64_t *cptr,
                                                              const int64_t *csrc, const double *G,
                                                              const double *b, double *z, double *delta,
                                                              const int32_t *done) {
    if (done != nullptr && *(volatile const int32_t *)done != 0) return;
    extern __shared__ double v[];
    const int4 it = items[blockIdx.x];
    const NodeMeta mt = meta[it.x];
    const int o = (int)mt.o;
    for (int p = threadIdx.x; p < o; p += blockDim.x)
        v[p] = b[idx[mt.ioff + p]] + gather_updates(cptr, csrc, delta, mt.coff + p);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = it.y + warp; r < it.z; r += kThreads / 32) {
        const double *row = G + mt.goff + (int64_t)r * o;
        double acc = 0.0;
#pragma unroll 4
        for (int c = lane; c < o; c += 32) acc += row[c] * v[c];
        acc = warp_sum(acc);
        if (lane == 0) {
            if (r < o) z[idx[mt.ioff + r]] = acc;
            else delta[mt.doff + (r - o)] = acc + gather_updates(cptr, csrc, delta, mt.coff + r);
        }
    }
}

__global__ void __launch_bounds__(kThreads) nd_backward_kernel(const int4 *items, const NodeMeta *meta,
                                                               const int32_t *idx, const double *H,
                                                               const double *z, double *x,
                                                               const int32_t *done) {
    if (done != nullptr && *(volatile const int32_t *)done != 0) return;
    extern __shared__ double w[];
    const int4 it = items[blockIdx.x];
    const NodeMeta mt = meta[it.x];
    const int o = (int)mt.o, m = (int)mt.m;
    for (int p = threadIdx.x; p < m; p += blockDim.x) {
        const int32_t g = idx[mt.ioff + p];
        w[p] = p < o ? z[g] : x[g];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = it.y + warp; r < it.z; r += kThreads / 32) {
        const double *row = H + mt.hoff + (int64_t)r * m;
        double acc = 0.0;
#pragma unroll 4
        for (int c = lane; c < m; c += 32) acc += row[c] * w[c];
        acc = warp_sum(acc);
        if (lane == 0) x[idx[mt.ioff + r]] = acc;
    }
}

constexpr size_t kMaxShm = 200 * 1024;

template <typename K>
int shm_for(K kern, int32_t n_values, size_t *shm) {
    if (n_values < 0) return PBTE_ERR_ARG;
    *shm = (size_t)(n_values > 0 ? n_values : 1) * sizeof(double);
    if (*shm > kMaxShm) return PBTE_ERR_UNSUPPORTED;
    if (*shm > 48 * 1024 &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxShm) != cudaSuccess)
        return PBTE_ERR_CUDA;
    return PBTE_OK;
}

}  // namespace

extern "C" int pbte_nd_forward(const int32_t *items, int32_t n_items, const int64_t *meta, const int32_t *idx,
                               const int64_t *cptr, const int64_t *csrc, const double *G, const double *b,
                               double *z, double *delta, int32_t max_own, const int32_t *done, void *stream) {
    if (!items || !meta || !idx || !cptr || !csrc || !G || !b || !z || !delta || n_items < 0) return PBTE_ERR_ARG;
    if (n_items == 0) return PBTE_OK;
    size_t shm = 0;
    int rc = shm_for(nd_forward_kernel, max_own, &shm);
    if (rc) return rc;
    nd_forward_kernel<<<n_items, kThreads, shm, reinterpret_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const int4 *>(items), reinterpret_cast<const NodeMeta *>(meta), idx, cptr, csrc, G, b, z,
        delta, done);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

extern "C" int pbte_nd_backward(const int32_t *items, int32_t n_items, const int64_t *meta, const int32_t *idx,
                                const double *H, const double *z, double *x, int32_t max_front, const int32_t *done,
                                void *stream) {
    if (!items || !meta || !idx || !H || !z || !x || n_items < 0) return PBTE_ERR_ARG;
    if (n_items == 0) return PBTE_OK;
    size_t shm = 0;
    int rc = shm_for(nd_backward_kernel, max_front, &shm);
    if (rc) return rc;
    nd_backward_kernel<<<n_items, kThreads, shm, reinterpret_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const int4 *>(items), reinterpret_cast<const NodeMeta *>(meta), idx, H, z, x, done);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}
