// Classical Gram-Schmidt applied twice (pybte/krylov.py:201-210) for a
// Krylov basis Q[0..j] of long vectors (n ~ 1e5..1e6) and few rows.
//
//   c1 = Q w;  w -= Q^T c1;  c2 = Q w;  w -= Q^T c2;  h = c1 + c2;  h[j+1] = ||w||
//
// Three launches: pass 1 (c1), pass 2 (update by c1, then c2 and h), and the
// last update fused with the norm.  A block owns chunks of kT * kE
// consecutive entries; a thread keeps its kE entries of w in registers while
// the rows stream past in batches of kRB (so registers do not grow with the
// row count, and a batch's loads are in flight together).  Per row, each
// warp reduces with shuffles and the block's warps are added in warp order
// into one partial per (block, row).  The last block to finish (a fence,
// then a ticket from an atomic counter -- nothing waits on it) adds the
// block partials per row in block order with a fixed warp tree, so the result
// is deterministic and no separate reduction launch is needed.
//
// Two storage types: FP64 basis (V = double, the FP64 GMRES) and FP32 basis
// (V = float, the inner GMRES of the mixed-precision solve, whose operator
// is an FP32 sweep).  GB300 runs FP64 at 1/64 of the FP32 rate, and the FP64
// products made the FP64 basis the largest cost of an inner Arnoldi column;
// in the FP32 form the products, the per-thread and the warp sums are FP32
// and only the block partials and the cross-block sums are FP64.
#include <algorithm>

#include <cuda_runtime.h>

#include "pbte_internal.cuh"

namespace {

constexpr int kT = 256;
constexpr int kWarps = kT / 32;
constexpr int kE = 4;              // entries per thread per chunk
constexpr int kRB = 8;             // rows per batch
constexpr int kMaxBlocks = 1216;   // 8 x 152 SMs
constexpr int kMaxBasis = PBTE_MAX_BASIS;
constexpr long long kHead = 8 + 2LL * kMaxBasis;

template <typename V>
__device__ __forceinline__ V warp_sum(V v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__host__ __device__ inline int row_stride(int rows) { return (rows + 7) / 8 * 8; }

// Scratch layout (doubles): the ticket counter (one unsigned in the first
// 8-byte slot, kept at zero between calls), c1[kMaxBasis], c2[kMaxBasis],
// then the block partials part[block][stride] with stride = rows rounded up
// to 8.  The head does not move with the row count, so the ticket stays put
// while a basis grows.
struct Scratch {
    double *part, *c1, *c2;
    unsigned int *ticket;
    int stride;
};

__host__ __device__ inline Scratch scratch_of(double *s, int rows) {
    Scratch r;
    r.ticket = reinterpret_cast<unsigned int *>(s);
    r.c1 = s + 8;
    r.c2 = r.c1 + kMaxBasis;
    r.part = r.c2 + kMaxBasis;
    r.stride = row_stride(rows);
    return r;
}

inline long long scratch_needed(int rows) { return kHead + (long long)kMaxBlocks * row_stride(rows); }

// dynamic shared memory of a CGS2 pass: per-warp row sums wsum[kWarps][stride]
// and the row coefficients csh[stride]; the norm pass's last block reuses it
// for the Givens staging (3 (rows + 1) doubles <= kWarps * stride)
template <typename V>
inline size_t pass_shm(int rows) {
    return (size_t)kWarps * row_stride(rows) * sizeof(double) + (size_t)row_stride(rows) * sizeof(V);
}

// After the block's partials are stored: one fence and one ticket per
// block.  Returns true in the one block that arrives last (which then owns
// the cross-block sums).
__device__ __forceinline__ bool last_block(unsigned int *ticket) {
    __shared__ bool is_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        is_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (is_last) __threadfence();
    return is_last;
}

// sum over blocks of part[b][k] in a fixed order: warp wid handles rows
// wid, wid + kWarps, ...; lane l adds blocks l, l + 32, ... (loads of a
// round of 8 first) then the warp tree.  Writes out[k] (and out_plus[k] =
// out[k] + add[k] when given), or the square root when `root`.
__device__ void finish_rows(const double *part, int stride, int rows, double *out, const double *add,
                            double *out_plus, bool root) {
    const int lane = threadIdx.x % 32, wid = threadIdx.x / 32;
    const int nb = gridDim.x;
    for (int k = wid; k < rows; k += kWarps) {
        double s = 0.0;
        for (int b0 = 0; b0 < nb; b0 += 256) {
            double v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int b = b0 + lane + 32 * i;
                v[i] = b < nb ? __ldcg(part + (size_t)b * stride + k) : 0.0;
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) s += v[i];
        }
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

// x[e] -= sum_k Q[k][t_e] c[k] over the rows, batches of kRB loads in flight
template <typename V>
__device__ __forceinline__ void subtract_rows(const V *__restrict__ Q, long long ldq, int rows, const V *csh,
                                              long long base, long long n, V (&x)[kE]) {
    int k = 0;
    for (; k + kRB <= rows; k += kRB) {
        V qv[kRB][kE];
#pragma unroll
        for (int r = 0; r < kRB; ++r)
#pragma unroll
            for (int e = 0; e < kE; ++e) {
                const long long t = base + (long long)e * kT;
                qv[r][e] = t < n ? Q[(k + r) * ldq + t] : V(0);
            }
#pragma unroll
        for (int r = 0; r < kRB; ++r) {
            const V ck = csh[k + r];
#pragma unroll
            for (int e = 0; e < kE; ++e) x[e] -= qv[r][e] * ck;
        }
    }
    for (; k < rows; ++k) {
        const V ck = csh[k];
#pragma unroll
        for (int e = 0; e < kE; ++e) {
            const long long t = base + (long long)e * kT;
            if (t < n) x[e] -= Q[k * ldq + t] * ck;
        }
    }
}

// wsum[wid * stride + k] += warp sum of sum_e Q[k][t_e] x[e], for every row
template <typename V>
__device__ __forceinline__ void dot_rows(const V *__restrict__ Q, long long ldq, int rows, long long base,
                                         long long n, const V (&x)[kE], double *wsum, int stride) {
    const int lane = threadIdx.x % 32, wid = threadIdx.x / 32;
    double *ws = wsum + (size_t)wid * stride;
    int k = 0;
    for (; k + kRB <= rows; k += kRB) {
        V a[kRB];
#pragma unroll
        for (int r = 0; r < kRB; ++r) {
            a[r] = V(0);
#pragma unroll
            for (int e = 0; e < kE; ++e) {
                const long long t = base + (long long)e * kT;
                if (t < n) a[r] += Q[(k + r) * ldq + t] * x[e];
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int r = 0; r < kRB; ++r) a[r] += __shfl_xor_sync(0xffffffffu, a[r], o);
        if (lane == 0)
#pragma unroll
            for (int r = 0; r < kRB; ++r) ws[k + r] += (double)a[r];
    }
    for (; k < rows; ++k) {
        V a = V(0);
#pragma unroll
        for (int e = 0; e < kE; ++e) {
            const long long t = base + (long long)e * kT;
            if (t < n) a += Q[k * ldq + t] * x[e];
        }
        a = warp_sum(a);
        if (lane == 0) ws[k] += (double)a;
    }
}

// A GMRES Givens step (gmres_givens_kernel's arguments) for the last block of
// the norm pass to run once h[j+1] is known; j < 0: none.  bounded != 0:
// tol_abs holds [tol_abs, enough] and state [stop, columns, products before
// the cycle, reached] -- pybte's bounded extension (krylov.py:332-338).
struct GivensStep {
    int j;
    const double *h;
    double *R;
    int ldr;
    double *cs, *sn, *gam;
    const double *tol_abs;
    int32_t *state;
    double *hist;
    int bounded;
};

__device__ void givens_column(const GivensStep &a, double *stage);

// MODE 0: x = w (or, with uout, x = qj - (uout - g), stored into w), then
//         out[k] = sum_t Q[k][t] x[t].
// MODE 1: x = w - Q^T c, stored into w, then out[k] = Q[k] . x and
//         out_plus[k] = out[k] + add[k].
// MODE 2: x = w - Q^T c, stored into w, then out[0] = ||x||.
template <typename V, int MODE>
__global__ void __launch_bounds__(kT) cgs2_pass_kernel(const V *__restrict__ Q, long long ldq, int rows,
                                                       V *__restrict__ w, const double *__restrict__ c, long long n,
                                                       double *scratch, double *out, const double *add,
                                                       double *out_plus, const V *__restrict__ qj,
                                                       const double *__restrict__ uout,
                                                       const double *__restrict__ g, const int32_t *done,
                                                       GivensStep gv) {
    extern __shared__ __align__(16) unsigned char cg_smem[];
    // a device-side stop flag set by an earlier launch: every block returns
    // before touching the ticket, which therefore stays at zero
    if (done != nullptr && *(volatile const int32_t *)done != 0) return;
    const Scratch S = scratch_of(scratch, rows);
    const int stride = S.stride;
    double *wsum = reinterpret_cast<double *>(cg_smem);              // [kWarps][stride]
    V *csh = reinterpret_cast<V *>(wsum + (size_t)kWarps * stride);    // [stride]
    const int nrow = MODE == 2 ? 1 : rows;
    for (int i = threadIdx.x; i < kWarps * stride; i += kT) wsum[i] = 0.0;
    if (MODE > 0)
        for (int i = threadIdx.x; i < rows; i += kT) csh[i] = (V)c[i];
    __syncthreads();
    const long long chunk = (long long)kT * kE;
    const long long nchunk = (n + chunk - 1) / chunk;
    V nrm = V(0);
    for (long long ch = blockIdx.x; ch < nchunk; ch += gridDim.x) {
        const long long base = ch * chunk + threadIdx.x;
        V x[kE];
#pragma unroll
        for (int e = 0; e < kE; ++e) {
            const long long t = base + (long long)e * kT;
            if (t >= n) {
                x[e] = V(0);
            } else if (MODE == 0 && uout) {
                double y = uout[t];
                if (g) y -= g[t];
                x[e] = (V)((double)qj[t] - y);
                w[t] = x[e];
            } else {
                x[e] = w[t];
            }
        }
        if (MODE > 0) {
            subtract_rows<V>(Q, ldq, rows, csh, base, n, x);
#pragma unroll
            for (int e = 0; e < kE; ++e) {
                const long long t = base + (long long)e * kT;
                if (t < n) w[t] = x[e];
            }
        }
        if (MODE < 2) {
            dot_rows<V>(Q, ldq, rows, base, n, x, wsum, stride);
        } else {
#pragma unroll
            for (int e = 0; e < kE; ++e) nrm += x[e] * x[e];
        }
    }
    if (MODE == 2) {
        nrm = warp_sum(nrm);
        if (threadIdx.x % 32 == 0) wsum[(threadIdx.x / 32) * stride] = (double)nrm;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nrow; k += kT) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < kWarps; ++q) s += wsum[q * stride + k];
        S.part[(size_t)blockIdx.x * stride + k] = s;
    }
    if (last_block(S.ticket)) {
        finish_rows(S.part, stride, nrow, out, add, out_plus, MODE == 2);
        if (threadIdx.x == 0) *S.ticket = 0u;
        if (MODE == 2 && gv.j >= 0) {
            // the rotation of this column, now that h[j+1] is written
            __syncthreads();
            if (threadIdx.x < 32) givens_column(gv, wsum);
        }
    }
}

template <typename K>
int allow_shm(K kern, size_t shm) {
    if (shm <= 48 * 1024) return PBTE_OK;
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm) == cudaSuccess
               ? PBTE_OK
               : PBTE_ERR_CUDA;
}

// uout == nullptr: CGS2 of w in place.  Otherwise pass 1 first forms
// w = Q[rows-1] - (uout - g) (the Arnoldi product of the newest basis vector).
// done (optional): every launch returns at once while *done != 0.
template <typename V>
int cgs2(const V *Q, int64_t ldq, int32_t rows, V *w, int64_t n, double *h, double *scratch, int64_t scratch_len,
         const double *uout, const double *g, const int32_t *done, void *stream,
         GivensStep gv = GivensStep{-1, nullptr, nullptr, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0}) {
    const GivensStep none{-1, nullptr, nullptr, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0};
    if (!Q || !w || !h || !scratch || rows < 1 || rows > kMaxBasis || n < 1 || ldq < n) return PBTE_ERR_ARG;
    if (scratch_len < scratch_needed(rows)) return PBTE_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const Scratch S = scratch_of(scratch, rows);
    const V *qj = Q + (size_t)(rows - 1) * ldq;
    const long long nchunk = (n + (long long)kT * kE - 1) / ((long long)kT * kE);
    const int nb = (int)std::min<long long>(nchunk, kMaxBlocks);
    const size_t shm = pass_shm<V>(rows);
    if (allow_shm(cgs2_pass_kernel<V, 0>, shm) || allow_shm(cgs2_pass_kernel<V, 1>, shm) ||
        allow_shm(cgs2_pass_kernel<V, 2>, shm))
        return PBTE_ERR_CUDA;
    cgs2_pass_kernel<V, 0><<<nb, kT, shm, s>>>(Q, ldq, rows, w, nullptr, n, scratch, S.c1, nullptr, nullptr, qj,
                                               uout, g, done, none);
    cgs2_pass_kernel<V, 1><<<nb, kT, shm, s>>>(Q, ldq, rows, w, S.c1, n, scratch, S.c2, S.c1, h,   // h = c1 + c2
                                               nullptr, nullptr, nullptr, done, none);
    cgs2_pass_kernel<V, 2><<<nb, kT, shm, s>>>(Q, ldq, rows, w, S.c2, n, scratch, h + rows, nullptr, nullptr,
                                               nullptr, nullptr, nullptr, done, gv);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

// Column j of a restart cycle on the device (gmres_full's host loop,
// pybte/krylov.py:211-235): the earlier rotations applied to the Hessenberg
// column h[0..j+1], the new rotation from hypot(h_j, h_j+1), the column of
// R, the residual estimates gam, and the stop state: state[0] = 1 when
// |gam[j+1]| <= tol_abs[0], 3 when pybte's bounded extension ends the solve
// (bounded steps only: the first product whose residual is <= tol_abs[1] sets
// state[3] = its index n among the run's products, n = state[2] + j + 1, and
// the solve halts once n - state[3] > max(64, state[3] / 4)), 2 when
// h[j+1] == 0 (breakdown); in that order of precedence, as gmres_full tests
// them.  state[1] = columns done, hist[j] = |gam[j+1]|.  Run by one warp;
// nothing runs once state[0] != 0.  stage: 3 (j + 2) doubles of shared memory.
__device__ void givens_column(const GivensStep &a, double *stage) {
    // the column and the rotations are staged in shared memory by the warp
    // (independent loads), then lane 0 runs the sequential rotations
    double *col = stage, *c_s = stage + (a.j + 2), *s_s = c_s + (a.j + 1);
    const int j = a.j;
    if (*(volatile const int32_t *)a.state != 0) return;
    for (int i = threadIdx.x; i <= j + 1; i += 32) col[i] = a.h[i];
    for (int i = threadIdx.x; i < j; i += 32) {
        c_s[i] = a.cs[i];
        s_s[i] = a.sn[i];
    }
    __syncwarp();
    if (threadIdx.x == 0) {
        const double hn = col[j + 1];
        double x = col[0];
        for (int i = 0; i < j; ++i) {
            const double b = col[i + 1];
            col[i] = c_s[i] * x + s_s[i] * b;
            x = -s_s[i] * x + c_s[i] * b;
        }
        col[j] = x;
        const double d = hypot(col[j], col[j + 1]);
        double c = 1.0, sv = 0.0;
        if (d != 0.0) {
            c = col[j] / d;
            sv = col[j + 1] / d;
        }
        a.cs[j] = c;
        a.sn[j] = sv;
        col[j] = d;
        const double gj = a.gam[j];
        a.gam[j + 1] = -sv * gj;
        a.gam[j] = c * gj;
        const double res = fabs(-sv * gj);
        a.hist[j] = res;
        a.state[1] = j + 1;
        bool halt = false;
        if (a.bounded) {
            const int n = a.state[2] + j + 1;
            if (a.state[3] < 0 && res <= a.tol_abs[1]) a.state[3] = n;
            const int reached = a.state[3];
            halt = reached >= 0 && n - reached > max(64, reached / 4);
        }
        if (res <= a.tol_abs[0]) a.state[0] = 1;
        else if (halt) a.state[0] = 3;
        else if (hn == 0.0) a.state[0] = 2;
    }
    __syncwarp();
    for (int i = threadIdx.x; i <= j; i += 32) a.R[(size_t)j * a.ldr + i] = col[i];
}

__global__ void gmres_givens_kernel(GivensStep a) {
    extern __shared__ double gstage[];
    givens_column(a, gstage);
}

// q_{j+1} = w / h[j+1] into row j+1 of the basis, and widened into the
// operator's FP64 input for the next product; nothing once state[0] != 0.
template <typename V>
__global__ void gmres_next_basis_kernel(int j, const V *__restrict__ w, const double *__restrict__ h,
                                        V *__restrict__ Q, long long ldq, double *__restrict__ uin, long long n,
                                        const int32_t *state) {
    if (*(volatile const int32_t *)state != 0) return;
    const V hn = (V)h[j + 1];
    V *q = Q + (size_t)(j + 1) * ldq;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const V v = w[t] / hn;
        q[t] = v;
        uin[t] = (double)v;
    }
}

template <typename V>
int next_basis(int32_t j, const V *w, const double *h, V *Q, int64_t ldq, double *uin, int64_t n,
               const int32_t *state, void *stream) {
    if (j < 0 || j + 1 >= kMaxBasis || !w || !h || !Q || !uin || !state || n < 1 || ldq < n) return PBTE_ERR_ARG;
    const int th = 256;
    const int bl = (int)std::min<long long>((n + th - 1) / th, 152 * 8);
    gmres_next_basis_kernel<V><<<bl, th, 0, reinterpret_cast<cudaStream_t>(stream)>>>(j, w, h, Q, ldq, uin, n, state);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

}  // namespace

namespace pbte {
// pbte_arnoldi_column_f32 then pbte_gmres_givens for column j = rows - 1,
// the rotation run by the last block of the norm pass (one launch fewer)
int arnoldi_column_givens_f32(const float *Q, int64_t ldq, int32_t rows, const double *uout, const double *g,
                              float *w, int64_t n, double *h, double *scratch, int64_t scratch_len, double *R,
                              int32_t ldr, double *cs, double *sn, double *gam, const double *tol_abs,
                              int32_t *state, double *hist, cudaStream_t s) {
    const int j = rows - 1;
    if (!uout || j < 0 || j + 1 > kMaxBasis || ldr < j + 1 || !h || !R || !cs || !sn || !gam || !tol_abs ||
        !state || !hist)
        return PBTE_ERR_ARG;
    return cgs2<float>(Q, ldq, rows, w, n, h, scratch, scratch_len, uout, g, state, s,
                       GivensStep{j, h, R, ldr, cs, sn, gam, tol_abs, state, hist, 0});
}
}  // namespace pbte

// h[0..rows-1] = c1 + c2 and h[rows] = ||w|| after the two passes; `scratch`
// holds scratch_len >= PBTE_CGS2_SCRATCH_ROWS(rows) doubles, zero before the
// first call.  rows <= PBTE_MAX_BASIS.
extern "C" int pbte_cgs2(const double *Q, int64_t ldq, int32_t rows, double *w, int64_t n, double *h,
                         double *scratch, int64_t scratch_len, void *stream) {
    return cgs2<double>(Q, ldq, rows, w, n, h, scratch, scratch_len, nullptr, nullptr, nullptr, stream);
}

extern "C" int pbte_cgs2_f32(const float *Q, int64_t ldq, int32_t rows, float *w, int64_t n, double *h,
                             double *scratch, int64_t scratch_len, void *stream) {
    return cgs2<float>(Q, ldq, rows, w, n, h, scratch, scratch_len, nullptr, nullptr, nullptr, stream);
}

extern "C" int pbte_arnoldi_column(const double *Q, int64_t ldq, int32_t rows, const double *uout, const double *g,
                                   double *w, int64_t n, double *h, double *scratch, int64_t scratch_len,
                                   const int32_t *done, void *stream) {
    if (!uout) return PBTE_ERR_ARG;
    return cgs2<double>(Q, ldq, rows, w, n, h, scratch, scratch_len, uout, g, done, stream);
}

extern "C" int pbte_arnoldi_column_f32(const float *Q, int64_t ldq, int32_t rows, const double *uout,
                                       const double *g, float *w, int64_t n, double *h, double *scratch,
                                       int64_t scratch_len, const int32_t *done, void *stream) {
    if (!uout) return PBTE_ERR_ARG;
    return cgs2<float>(Q, ldq, rows, w, n, h, scratch, scratch_len, uout, g, done, stream);
}

static int givens_launch(const GivensStep &a, void *stream) {
    if (a.j < 0 || a.j + 1 > kMaxBasis || a.ldr < a.j + 1 || !a.h || !a.R || !a.cs || !a.sn || !a.gam ||
        !a.tol_abs || !a.state || !a.hist)
        return PBTE_ERR_ARG;
    const size_t shm = (size_t)3 * (a.j + 2) * sizeof(double);
    if (allow_shm(gmres_givens_kernel, shm)) return PBTE_ERR_CUDA;
    gmres_givens_kernel<<<1, 32, shm, reinterpret_cast<cudaStream_t>(stream)>>>(a);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

extern "C" int pbte_gmres_givens(int32_t j, const double *h, double *R, int32_t ldr, double *cs, double *sn,
                                 double *gam, const double *tol_abs, int32_t *state, double *hist, void *stream) {
    return givens_launch(GivensStep{j, h, R, ldr, cs, sn, gam, tol_abs, state, hist, 0}, stream);
}

extern "C" int pbte_gmres_givens_bounded(int32_t j, const double *h, double *R, int32_t ldr, double *cs,
                                         double *sn, double *gam, const double *tol2, int32_t *state,
                                         double *hist, void *stream) {
    return givens_launch(GivensStep{j, h, R, ldr, cs, sn, gam, tol2, state, hist, 1}, stream);
}

extern "C" int pbte_arnoldi_column_givens(const double *Q, int64_t ldq, int32_t rows, const double *uout,
                                          const double *g, double *w, int64_t n, double *h, double *scratch,
                                          int64_t scratch_len, double *R, int32_t ldr, double *cs, double *sn,
                                          double *gam, const double *tol2, int32_t *state, double *hist,
                                          int32_t bounded, void *stream) {
    const int j = rows - 1;
    if (!uout || j < 0 || j + 1 > kMaxBasis || ldr < j + 1 || !h || !R || !cs || !sn || !gam || !tol2 || !state ||
        !hist)
        return PBTE_ERR_ARG;
    return cgs2<double>(Q, ldq, rows, w, n, h, scratch, scratch_len, uout, g, state, stream,
                        GivensStep{j, h, R, ldr, cs, sn, gam, tol2, state, hist, bounded ? 1 : 0});
}

extern "C" int pbte_gmres_next_basis(int32_t j, const double *w, const double *h, double *Q, int64_t ldq,
                                     double *uin, int64_t n, const int32_t *state, void *stream) {
    return next_basis<double>(j, w, h, Q, ldq, uin, n, state, stream);
}

extern "C" int pbte_gmres_next_basis_f32(int32_t j, const float *w, const double *h, float *Q, int64_t ldq,
                                         double *uin, int64_t n, const int32_t *state, void *stream) {
    return next_basis<float>(j, w, h, Q, ldq, uin, n, state, stream);
}

static_assert(PBTE_CGS2_SCRATCH_ROWS(64) == kHead + (long long)kMaxBlocks * 64, "scratch size");
static_assert(PBTE_CGS2_SCRATCH >= PBTE_CGS2_SCRATCH_ROWS(64), "scratch size");
