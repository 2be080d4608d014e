// Device solve of the GSIS trace system with a nested-dissection
// multifrontal factorisation (factors built on the host by
// pbte_gb300/trace_nd.py; replaces the SuperLU triangular solves of
// pybte/acceleration/global_solve.py:189-195).
//
// Per tree node (front) the host stores
//   G = [L11^-1 P ; -L21 L11^-1 P]   (m x o)
//   H = [U11^-1, -U11^-1 U12]        (o x m)
// column-major (G^T and H^T row-major) for its o own and m - o boundary
// unknowns.  The forward sweep runs the nodes by height (leaves first): the
// node's own right-hand side is the original one plus its children's
// boundary updates, y = G_top v goes to z, and its own boundary update
// G_bot v plus the children's updates to those unknowns goes to its delta
// slots.  The backward sweep (root first) forms x_own = H [z_own ; x_bnd].
// One thread block per work item (a node, a run of output rows and a count
// kc of column groups, laid out by the host so that a height is about a
// wave of blocks); the input vector and the children's updates are gathered
// into shared memory by all threads first, then a thread per output row and
// column group.  FP64 throughput bounds this solve on GB300, so every
// factor entry costs one FMA and no warp reductions are made.  Sums are in
// a fixed order, so the solve is deterministic.
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

// The item's output rows r0..r1 of a factor stored column-major (entry
// (row r, column c) at mat[off + c * ld + r]) against a vector in shared
// memory.  Thread t takes row r0 + t % (256 / kc) and the t / (256 / kc)-th
// of kc contiguous column chunks (kc a power of two up to 64): a warp reads
// runs of consecutive rows of a column (coalesced), each factor entry costs
// one FP64 FMA, and eight loads per thread are issued before their
// products.  The first eight are issued when the item is read, before the
// kernel gathers the vector, so they overlap its dependent loads.  The kc
// partials of a row are summed by a fixed pairwise tree, so the sums run in
// a fixed order.  Warps with no row of the item skip the columns.
struct ItemRows {
    int kc, rp, lr, grp, r, c0, c1;
    bool ok, live;
    const double *col;
    int64_t ld;
    double g[8];

    __device__ __forceinline__ ItemRows(const double *__restrict__ mat, int64_t off, int64_t ld_, int len,
                                        const int4 it) {
        kc = (it.w >= 1 && it.w <= 64 && (it.w & (it.w - 1)) == 0) ? it.w : 1;
        rp = kThreads / kc;
        lr = threadIdx.x % rp;
        grp = threadIdx.x / rp;
        r = it.y + lr;
        ok = r < it.z;
        live = it.y + (lr & ~31) < it.z;
        const int per = (len + kc - 1) / kc;
        c0 = min(len, grp * per);
        c1 = min(len, c0 + per);
        ld = ld_;
        col = mat + off + r;
    }

    __device__ __forceinline__ void load(int c) {
#pragma unroll
        for (int j = 0; j < 8; ++j) g[j] = (live && ok && c + j < c1) ? __ldg(col + (int64_t)(c + j) * ld) : 0.0;
    }

    // the row's sum, valid in the threads of group 0; every thread calls it
    __device__ __forceinline__ double sum(const double *vec, double *part) {
        double acc = 0.0;
        if (live) {
            for (int c = c0; c < c1; c += 8) {
                load(c);
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (c + j < c1) acc = fma(g[j], vec[c + j], acc);
            }
        }
        if (kc > 1) {
            part[threadIdx.x] = acc;
            for (int half = kc >> 1; half > 0; half >>= 1) {
                __syncthreads();
                if (grp < half) part[threadIdx.x] += part[threadIdx.x + half * rp];
            }
            __syncthreads();
            acc = part[threadIdx.x];
        }
        return acc;
    }

    __device__ __forceinline__ bool stores() const { return ok && grp == 0; }
};

__global__ void __launch_bounds__(kThreads, 6) nd_forward_kernel(const int4 *__restrict__ items,
                                                                 const NodeMeta *__restrict__ meta,
                                                                 const int32_t *__restrict__ idx,
                                                                 const int64_t *__restrict__ cptr,
                                                                 const int64_t *__restrict__ csrc,
                                                                 const double *__restrict__ G,
                                                                 const double *__restrict__ b,
                                                                 double *__restrict__ z, double *delta,
                                                                 const int32_t *done) {
    const int4 it = items[blockIdx.x];
    if (done != nullptr && *(volatile const int32_t *)done != 0) return;
    extern __shared__ double v[];  // the o inputs
    __shared__ double part[kThreads];
    const NodeMeta mt = meta[it.x];
    const int o = (int)mt.o;
    ItemRows rows(G, mt.goff, mt.m, o, it);  // G^T: o columns of m entries
    // the row's destination (own rows) or its children's updates (boundary
    // rows), fetched alongside the vector
    int32_t dst = 0;
    double upd = 0.0;
    if (rows.stores()) {
        if (rows.r < o) dst = idx[mt.ioff + rows.r];
        else upd = gather_updates(cptr, csrc, delta, mt.coff + rows.r);
    }
    for (int p = threadIdx.x; p < o; p += blockDim.x)
        v[p] = b[idx[mt.ioff + p]] + gather_updates(cptr, csrc, delta, mt.coff + p);
    __syncthreads();
    const double acc = rows.sum(v, part);
    if (rows.stores()) {
        if (rows.r < o) z[dst] = acc;
        else delta[mt.doff + (rows.r - o)] = acc + upd;
    }
}

__global__ void __launch_bounds__(kThreads, 6) nd_backward_kernel(const int4 *__restrict__ items,
                                                                  const NodeMeta *__restrict__ meta,
                                                                  const int32_t *__restrict__ idx,
                                                                  const double *__restrict__ H,
                                                                  const double *__restrict__ z, double *x,
                                                                  const int32_t *done) {
    const int4 it = items[blockIdx.x];
    if (done != nullptr && *(volatile const int32_t *)done != 0) return;
    extern __shared__ double w[];
    __shared__ double part[kThreads];
    const NodeMeta mt = meta[it.x];
    const int o = (int)mt.o, m = (int)mt.m;
    ItemRows rows(H, mt.hoff, mt.o, m, it);  // H^T: m columns of o entries
    const int32_t dst = rows.stores() ? idx[mt.ioff + rows.r] : 0;
    for (int p = threadIdx.x; p < m; p += blockDim.x) {
        const int32_t g = idx[mt.ioff + p];
        w[p] = p < o ? z[g] : x[g];
    }
    __syncthreads();
    const double acc = rows.sum(w, part);
    if (rows.stores()) x[dst] = acc;
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
