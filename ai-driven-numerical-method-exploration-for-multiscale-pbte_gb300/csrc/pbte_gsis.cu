// GSIS per-iteration kernels on the distribution (pybte/acceleration/):
// the third-order moment source (hot_source.py:29-58), the kinetic wall
// traces (global_solve.py:31-53) and the damped correction
// (correction.py:29-98).
//
// Each reads the whole distribution and is bound by GB300's FP64 pipe and
// by latency, so the angular sums are spread over direction chunks: a block
// of 32 (element, DOF) lanes x 8 chunks, each chunk summing every eighth
// ordinate, the chunks added in a fixed order through shared memory (the
// result does not depend on the launch).  A warp reads one ordinate's rows
// of 32 consecutive (element, DOF) entries: coalesced.
#include <cuda_runtime.h>

#include "pbte_device.cuh"

namespace pbte {
namespace {

constexpr int kLanes = 32, kChunks = 8;

// Angular sums out[k][t] = sum_d a_k(d) f[d][t] over t = i * NP + l.
// HOT: the four weights of the third-order moments, a_k = w c-polynomials;
// else the three moment weights w, c_x w, c_y w (then also the correction).
template <bool HOT>
__device__ __forceinline__ void weights(double cx, double cy, double dw, double (&a)[4]) {
    if constexpr (HOT) {
        a[0] = cx * (5.0 * cx * cx - 3.0) * dw;
        a[1] = cy * (5.0 * cx * cx - 1.0) * dw;
        a[2] = cx * (5.0 * cy * cy - 1.0) * dw;
        a[3] = cy * (5.0 * cy * cy - 3.0) * dw;
    } else {
        a[0] = dw;
        a[1] = cx * dw;
        a[2] = cy * dw;
        a[3] = 0.0;
    }
}

template <bool HOT>
__device__ __forceinline__ void chunk_sums(const double *vdf, const double *cx, const double *cy, const double *w,
                                           int ndir, size_t stride, int t, bool live, double (&acc)[4]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[k] = 0.0;
    if (!live) return;
    for (int d = threadIdx.y; d < ndir; d += kChunks) {
        const double f = vdf[(size_t)d * stride + t];
        double a[4];
        weights<HOT>(cx[d], cy[d], w[d], a);
        if constexpr (HOT) {
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[k] += a[k] * f;
        } else {
            // the reference's products: f w, c_x f w, c_y f w
            acc[0] += f * w[d];
            acc[1] += cx[d] * f * w[d];
            acc[2] += cy[d] * f * w[d];
        }
    }
}

// chunks 0..7 added in order by the chunk-0 thread of each lane
__device__ __forceinline__ void reduce_chunks(double (&acc)[4], int nk) {
    __shared__ double sm[kChunks][4][kLanes];
    for (int k = 0; k < nk; ++k) sm[threadIdx.y][k][threadIdx.x] = acc[k];
    __syncthreads();
    if (threadIdx.y == 0)
        for (int k = 0; k < nk; ++k) {
            double s = sm[0][k][threadIdx.x];
#pragma unroll
            for (int y = 1; y < kChunks; ++y) s += sm[y][k][threadIdx.x];
            acc[k] = s;
        }
}

// the four weights of every ordinate are formed once per block into shared
// memory (ws[k * ndir + d]); the FP64 pipe then only does the four sums
__global__ void __launch_bounds__(kLanes *kChunks) hot_moments_kernel(const double *vdf, const double *cx,
                                                                      const double *cy, const double *w, int ndir,
                                                                      int total, double *mk) {
    extern __shared__ double ws[];
    const int tid = threadIdx.y * kLanes + threadIdx.x;
    for (int d = tid; d < ndir; d += kLanes * kChunks) {
        double a[4];
        weights<true>(cx[d], cy[d], w[d], a);
#pragma unroll
        for (int k = 0; k < 4; ++k) ws[k * ndir + d] = a[k];
    }
    __syncthreads();
    const int t = blockIdx.x * kLanes + threadIdx.x;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    if (t < total)
        for (int d = threadIdx.y; d < ndir; d += kChunks) {
            const double f = vdf[(size_t)d * total + t];
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[k] += ws[k * ndir + d] * f;
        }
    reduce_chunks(acc, 4);
    if (threadIdx.y == 0 && t < total)
#pragma unroll
        for (int k = 0; k < 4; ++k) mk[(size_t)k * total + t] = acc[k];
}

// work rows 3..6 of element i from its four moment rows and the gradient
// operators gx, gy (compact form: area2 (xi_x Dx + eta_x Dy) ...)
__global__ void hot_contract_kernel(const double *mk, const CellRec<double> *cells, const double *ref, int nt,
                                    int NP, double tc5, double *work) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt * NP) return;
    const int i = t / NP, m = t % NP;
    const size_t total = (size_t)nt * NP;
    const CellRec<double> &r = cells[i];
    const double *Dx = ref + NP * NP, *Dy = ref + 2 * NP * NP;
    double pxx = 0.0, pxy = 0.0, pyy = 0.0;
    for (int l = 0; l < NP; ++l) {
        const size_t e = (size_t)i * NP + l;
        const double m0 = mk[e], m1 = mk[total + e], m2 = mk[2 * total + e], m3 = mk[3 * total + e];
        const double gx = r.area2 * (r.gxa * Dx[l * NP + m] + r.gxb * Dy[l * NP + m]);
        const double gy = r.area2 * (r.gya * Dx[l * NP + m] + r.gyb * Dy[l * NP + m]);
        pxx += gx * m0 + gy * m1;
        pxy += gx * m1 + gy * m2;
        pyy += gx * m2 + gy * m3;
    }
    double *o = work + (size_t)i * 7 * NP;
    o[3 * NP + m] = (pxx + 0.5 * pyy) * tc5;
    o[4 * NP + m] = 0.5 * pxy * tc5;
    o[5 * NP + m] = 0.5 * pxy * tc5;
    o[6 * NP + m] = (0.5 * pxx + pyy) * tc5;
}

// Kinetic wall traces: one block per wall face, threads over the ordinates,
// a fixed-order tree over the block for the 3 NF sums.
constexpr int kTraceThreads = 128;

__global__ void __launch_bounds__(kTraceThreads) wall_trace_kernel(const double *vdf, const double *tri_fc_fc,
                                                                   const double *cx, const double *cy,
                                                                   const double *w, int ndir, int nt, int NP, int NF,
                                                                   const int32_t *tri_list, const int32_t *lfc_list,
                                                                   double *out) {
    __shared__ double c[16 * kMaxNf];
    __shared__ double red[3 * kMaxNf][kTraceThreads];
    const int k = blockIdx.x;
    const int tri = tri_list[k], lfc = lfc_list[k];
    for (int e = threadIdx.x; e < NP * NF; e += blockDim.x) {
        const int l = e / NF, m = e % NF;
        c[e] = tri_fc_fc[(((size_t)l * NF + m) * nt + tri) * 3 + lfc];
    }
    __syncthreads();
    double acc[3 * kMaxNf];
    for (int q = 0; q < 3 * NF; ++q) acc[q] = 0.0;
    for (int d = threadIdx.x; d < ndir; d += blockDim.x) {
        const double *f = vdf + ((size_t)d * nt + tri) * NP;
        for (int m = 0; m < NF; ++m) {
            double tt = 0.0;
            for (int l = 0; l < NP; ++l) tt += f[l] * c[l * NF + m];
            acc[m] += tt * w[d];
            acc[NF + m] += cx[d] * tt * w[d];
            acc[2 * NF + m] += cy[d] * tt * w[d];
        }
    }
    for (int q = 0; q < 3 * NF; ++q) red[q][threadIdx.x] = acc[q];
    __syncthreads();
    for (int h = kTraceThreads / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            for (int q = 0; q < 3 * NF; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x < 3 * NF) out[(size_t)k * 3 * NF + threadIdx.x] = red[threadIdx.x][0];
}

// The correction's moments and coefficients: per (element, DOF) the
// distribution's T, q_x, q_y, the damped corrections l_T, l_qx, l_qy, the new
// moments, and the coefficients of the per-ordinate update in coef.
__global__ void __launch_bounds__(kLanes *kChunks) correct_moments_kernel(
    const double *vdf, const double *uq, const double *cx, const double *cy, const double *w, const double *tri_hmin,
    int ndir, int nt, int NP, double cv, double tau_r, double tau_thr, int use_hmin, double *ts, double *qxs,
    double *qys, double *coef) {
    const int total = nt * NP;
    const int t = blockIdx.x * kLanes + threadIdx.x;
    double acc[4];
    chunk_sums<false>(vdf, cx, cy, w, ndir, (size_t)total, t, t < total, acc);
    reduce_chunks(acc, 3);
    if (threadIdx.y != 0 || t >= total) return;
    const int i = t / NP, m = t % NP;
    const double tau_loc = use_hmin ? tau_r / tri_hmin[i] : tau_r;
    const double beta = fmin(tau_loc, tau_thr) / tau_loc;
    const double tv = acc[0] / cv, qxv = acc[1], qyv = acc[2];
    const double lt = (uq[(size_t)m * nt + i] - tv) * beta;
    const double lqx = (uq[(size_t)(NP + m) * nt + i] - qxv) * beta;
    const double lqy = (uq[(size_t)(2 * NP + m) * nt + i] - qyv) * beta;
    coef[t] = lt * cv / 4.0 / kPi;
    coef[total + t] = lqx;
    coef[2 * total + t] = lqy;
    ts[(size_t)m * nt + i] = lt + tv;
    qxs[(size_t)m * nt + i] = lqx + qxv;
    qys[(size_t)m * nt + i] = lqy + qyv;
}

// f[d][t] += eq + (c_x l_qx + c_y l_qy) drift, grid (t blocks, ordinate chunks)
__global__ void correct_update_kernel(double *vdf, const double *coef, const double *cx, const double *cy, int ndir,
                                      int total, double drift) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const double eq = coef[t], lqx = coef[total + t], lqy = coef[2 * total + t];
    for (int d = blockIdx.y; d < ndir; d += gridDim.y) {
        double *f = vdf + (size_t)d * total + t;
        *f = *f + eq + (cx[d] * lqx + cy[d] * lqy) * drift;
    }
}

}  // namespace

int launch_hot_source(pbte_ctx *c, const double *vdf, double tc5, double *work, cudaStream_t s) {
    const int total = c->n_tris * c->nd;
    const size_t shm = (size_t)4 * c->ndir * sizeof(double);
    if (shm > 48 * 1024) {
        if (shm > 200 * 1024) return PBTE_ERR_UNSUPPORTED;
        if (cudaFuncSetAttribute(hot_moments_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm) !=
            cudaSuccess)
            return PBTE_ERR_CUDA;
    }
    hot_moments_kernel<<<(total + kLanes - 1) / kLanes, dim3(kLanes, kChunks), shm, s>>>(
        vdf, c->d_cx, c->d_cy, c->d_w, c->ndir, total, c->d_gsis);
    const int th = 128;
    hot_contract_kernel<<<(total + th - 1) / th, th, 0, s>>>(c->d_gsis, c->d_cells64, c->d_ref64, c->n_tris, c->nd,
                                                            tc5, work);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

int launch_wall_trace(pbte_ctx *c, const double *vdf, const double *tri_fc_fc, int nk, const int32_t *tri_list,
                      const int32_t *lfc_list, double *out, cudaStream_t s) {
    if (nk <= 0) return PBTE_OK;
    if (c->nd > 16 || c->nf > kMaxNf) return PBTE_ERR_UNSUPPORTED;
    wall_trace_kernel<<<nk, kTraceThreads, 0, s>>>(vdf, tri_fc_fc, c->d_cx, c->d_cy, c->d_w, c->ndir, c->n_tris,
                                                   c->nd, c->nf, tri_list, lfc_list, out);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

int launch_correct(pbte_ctx *c, double *vdf, const double *uq, const double *tri_hmin, double tau_thr,
                   int use_hmin, double *ts, double *qxs, double *qys, double *temp, double *qx, double *qy,
                   cudaStream_t s) {
    const int total = c->n_tris * c->nd;
    correct_moments_kernel<<<(total + kLanes - 1) / kLanes, dim3(kLanes, kChunks), 0, s>>>(
        vdf, uq, c->d_cx, c->d_cy, c->d_w, tri_hmin, c->ndir, c->n_tris, c->nd, c->cv, c->tau_r, tau_thr, use_hmin,
        ts, qxs, qys, c->d_gsis);
    const double drift = c->tau_c / c->tau_n * 3.0 / 4.0 / kPi / c->vg / c->vg;
    const int th = 256;
    const int chunks = std::min(c->ndir, 16);
    correct_update_kernel<<<dim3((total + th - 1) / th, chunks), th, 0, s>>>(vdf, c->d_gsis, c->d_cx, c->d_cy, c->ndir,
                                                                           total, drift);
    return launch_element_integrals(c, ts, qxs, qys, temp, qx, qy, s);
}

}  // namespace pbte
