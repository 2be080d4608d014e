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

#include <algorithm>

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
                                                                      int total, double *mk,
                                                                      const int32_t *done) {
    if (stopped(done)) return;
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
                                    int NP, double tc5, double *work, const int32_t *done) {
    if (stopped(done)) return;
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
                                                                   double *out, const int32_t *done) {
    if (stopped(done)) return;
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
    double *qys, double *coef, const int32_t *done) {
    if (stopped(done)) return;
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
                                      int total, double drift, const int32_t *done) {
    if (stopped(done)) return;
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
        vdf, c->d_cx, c->d_cy, c->d_w, c->ndir, total, c->d_gsis, c->done);
    const int th = 128;
    hot_contract_kernel<<<(total + th - 1) / th, th, 0, s>>>(c->d_gsis, c->d_cells64, c->d_ref64, c->n_tris, c->nd,
                                                            tc5, work, c->done);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

int launch_wall_trace(pbte_ctx *c, const double *vdf, const double *tri_fc_fc, int nk, const int32_t *tri_list,
                      const int32_t *lfc_list, double *out, cudaStream_t s) {
    if (nk <= 0) return PBTE_OK;
    if (c->nd > 16 || c->nf > kMaxNf) return PBTE_ERR_UNSUPPORTED;
    wall_trace_kernel<<<nk, kTraceThreads, 0, s>>>(vdf, tri_fc_fc, c->d_cx, c->d_cy, c->d_w, c->ndir, c->n_tris,
                                                   c->nd, c->nf, tri_list, lfc_list, out, c->done);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

int launch_correct(pbte_ctx *c, double *vdf, const double *uq, const double *tri_hmin, double tau_thr,
                   int use_hmin, double *ts, double *qxs, double *qys, double *temp, double *qx, double *qy,
                   cudaStream_t s) {
    const int total = c->n_tris * c->nd;
    correct_moments_kernel<<<(total + kLanes - 1) / kLanes, dim3(kLanes, kChunks), 0, s>>>(
        vdf, uq, c->d_cx, c->d_cy, c->d_w, tri_hmin, c->ndir, c->n_tris, c->nd, c->cv, c->tau_r, tau_thr, use_hmin,
        ts, qxs, qys, c->d_gsis, c->done);
    const double drift = c->tau_c / c->tau_n * 3.0 / 4.0 / kPi / c->vg / c->vg;
    const int th = 256;
    const int chunks = std::min(c->ndir, 16);
    correct_update_kernel<<<dim3((total + th - 1) / th, chunks), th, 0, s>>>(vdf, c->d_gsis, c->d_cx, c->d_cy, c->ndir,
                                                                           total, drift, c->done);
    return launch_element_integrals(c, ts, qxs, qys, temp, qx, qy, s);
}


// ---------------------------------------------------------------------------
// Static condensation per GSIS iteration (pybte/acceleration/hot_source.py:74,
// global_solve.py:131-187, local_solve.py:16-26) on operator layouts made
// once at setup, field-major so that a warp reading one entry of consecutive
// (element, row) or (face, row) pairs makes one coalesced access:
//   inv_t[(q * n_tris + i) * M + p]           = inv(AA_SOL_i)[p][q]
//   ba1_t[(p * n_faces + f) * NF3 + r]        = BA_SOL of face f's first element
//   ba2_t[(p * n2 + k) * NF3 + r]             = BA_SOL of its second element
//   aa_trace_t[((il * NF3 + r) * n_tris + i) * M + p] = AA_TRACE_i[il][p][r]
// with M = 7 NP rows of an element's local unknowns and NF3 = 3 NF trace
// unknowns of a face.  Sums run in a fixed order, so results do not depend on
// the launch.
namespace {

__device__ __forceinline__ int per_block(int M) { return M >= 256 ? 1 : 256 / M; }

// aa_src[i][p] = sum_{q = 3NP}^{7NP-1} inv_t[q][i][p] * work_i[q], where rows
// 3..6 of work_i are the hot source of element i (hot_contract_kernel's
// arithmetic, formed in shared memory) and rows 0..2 are zero.
__global__ void __launch_bounds__(256) hot_apply_kernel(const double *mk, const CellRec<double> *cells,
                                                        const double *ref, int nt, int NP, double tc5,
                                                        const double *__restrict__ inv_t, double *aa_src,
                                                        const int32_t *done) {
    if (stopped(done)) return;
    extern __shared__ double hw[];   // [E][4 NP]
    const int M = 7 * NP, E = per_block(M);
    const int e = threadIdx.x / M, p = threadIdx.x % M;
    const int i = blockIdx.x * E + e;
    const bool live = e < E && i < nt;
    const size_t total = (size_t)nt * NP;
    if (live && p < NP) {
        const int m = p;
        const CellRec<double> &r = cells[i];
        const double *Dx = ref + NP * NP, *Dy = ref + 2 * NP * NP;
        double pxx = 0.0, pxy = 0.0, pyy = 0.0;
        for (int l = 0; l < NP; ++l) {
            const size_t el = (size_t)i * NP + l;
            const double m0 = mk[el], m1 = mk[total + el], m2 = mk[2 * total + el], m3 = mk[3 * total + el];
            const double gx = r.area2 * (r.gxa * Dx[l * NP + m] + r.gxb * Dy[l * NP + m]);
            const double gy = r.area2 * (r.gya * Dx[l * NP + m] + r.gyb * Dy[l * NP + m]);
            pxx += gx * m0 + gy * m1;
            pxy += gx * m1 + gy * m2;
            pyy += gx * m2 + gy * m3;
        }
        double *o = hw + e * 4 * NP;
        o[m] = (pxx + 0.5 * pyy) * tc5;
        o[NP + m] = 0.5 * pxy * tc5;
        o[2 * NP + m] = 0.5 * pxy * tc5;
        o[3 * NP + m] = (0.5 * pxx + pyy) * tc5;
    }
    __syncthreads();
    if (!live) return;
    const double *w = hw + e * 4 * NP;
    const double *a = inv_t + ((size_t)3 * NP * nt + i) * M + p;
    const size_t step = (size_t)nt * M;
    double acc = 0.0;
    for (int q = 0; q < 4 * NP; ++q) acc += a[q * step] * w[q];
    aa_src[(size_t)i * M + p] = acc;
}

// aa_src[i][p] = sum_{q = c0}^{c1-1} inv_t[q][i][p] * work[i][q] (any rows)
__global__ void __launch_bounds__(256) apply_inverse_kernel(int nt, int M, const double *__restrict__ inv_t,
                                                            const double *__restrict__ work, int c0, int c1,
                                                            double *aa_src, const int32_t *done) {
    if (stopped(done)) return;
    const int E = per_block(M);
    const int e = threadIdx.x / M, p = threadIdx.x % M;
    const int i = blockIdx.x * E + e;
    if (e >= E || i >= nt) return;
    const double *w = work + (size_t)i * M;
    const size_t step = (size_t)nt * M;
    const double *a = inv_t + (size_t)i * M + p;
    double acc = 0.0;
    for (int q = c0; q < c1; ++q) acc += a[q * step] * w[q];
    aa_src[(size_t)i * M + p] = acc;
}

// The trace right-hand side, one thread per (face, trace row r): the first
// element's BA_SOL AA_SRC, plus the second's (rows mirrored within each block
// of NF for a periodic pair walked the same way), then the wall rows imposed
// from the kinetic wall moments wall_mom[slot][3 NF] (global_solve.py:159-187):
// thermalising walls set T (and, variant B, q_x, q_y), diffuse adiabatic walls
// set T and the tangential projection of the wall heat flux.
__global__ void __launch_bounds__(256) trace_rhs_kernel(pbte_gsis_ops o, const double *__restrict__ aa_src,
                                                        const double *__restrict__ wall_mom, double *ffa,
                                                        const int32_t *done) {
    if (stopped(done)) return;
    const int NF = o.ndof_fc, NF3 = 3 * NF, M = 7 * o.ndof;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)o.n_faces * NF3) return;
    const int f = (int)(t / NF3), r = (int)(t % NF3);
    const double *src = aa_src + (size_t)o.tri1[f] * M;
    const double *b = o.ba1_t + (size_t)f * NF3 + r;
    const size_t step1 = (size_t)o.n_faces * NF3;
    double v = 0.0;
    for (int p = 0; p < M; ++p) v += b[p * step1] * src[p];
    const int k = o.slot2[f];
    if (k >= 0) {
        const int r2 = o.mirror2[k] ? (r / NF) * NF + (NF - 1 - r % NF) : r;
        const double *src2 = aa_src + (size_t)o.tri2[k] * M;
        const double *b2 = o.ba2_t + (size_t)k * NF3 + r2;
        const size_t step2 = (size_t)o.n2 * NF3;
        double c2 = 0.0;
        for (int p = 0; p < M; ++p) c2 += b2[p * step2] * src2[p];
        v += c2;
    }
    const int ws = o.wall_slot[f];
    if (ws >= 0) {
        const double *mw = wall_mom + (size_t)ws * NF3;
        const int blk = r / NF, rr = r % NF;
        if (o.wall_kind[f] == 1) {
            if (blk == 0) v = mw[rr] / o.cv;
            else if (o.variant == 1) v = mw[r];
        } else {
            const double nx = o.wall_nx[f], ny = o.wall_ny[f];
            const double qxb = mw[NF + rr], qyb = mw[2 * NF + rr];
            if (blk == 0) v = mw[rr] / o.cv;
            else if (blk == 1) v = qxb * (ny * ny) - qyb * (nx * ny);
            else v = -qxb * (nx * ny) + qyb * (nx * nx);
        }
    }
    ffa[t] = v;
}

// uq[p][i] = aa_src[i][p] + sum_il sum_r aa_trace_t[il][r][i][p] * u_trace[face(i, il)][r]
__global__ void __launch_bounds__(256) local_recover_kernel(pbte_gsis_ops o, const double *__restrict__ aa_src,
                                                            const double *__restrict__ u_trace, double *uq,
                                                            const int32_t *done) {
    if (stopped(done)) return;
    const int M = 7 * o.ndof, NF3 = 3 * o.ndof_fc, nt = o.n_tris, E = per_block(M);
    const int e = threadIdx.x / M, p = threadIdx.x % M;
    const int i = blockIdx.x * E + e;
    if (e >= E || i >= nt) return;
    double acc = 0.0;
    for (int il = 0; il < 3; ++il) {
        const double *u = u_trace + (size_t)o.tri_faces[i * 3 + il] * NF3;
        const double *a = o.aa_trace_t + ((size_t)il * NF3 * nt + i) * M + p;
        double s = 0.0;
        for (int r = 0; r < NF3; ++r) s += a[(size_t)r * nt * M] * u[r];
        acc += s;
    }
    uq[(size_t)p * nt + i] = aa_src[(size_t)i * M + p] + acc;
}

int elements_grid(int nt, int M, int *threads) {
    const int E = M >= 256 ? 1 : 256 / M;
    *threads = E * M;
    return (nt + E - 1) / E;
}

bool ops_ok(const pbte_gsis_ops *o) {
    return o && o->n_tris > 0 && o->n_faces > 0 && o->ndof > 0 && o->ndof <= 15 && o->ndof_fc > 0 &&
           o->ndof_fc <= kMaxNf && o->inv_t && o->ba1_t && o->tri1 && o->slot2 && o->wall_slot && o->wall_kind &&
           o->aa_trace_t && o->tri_faces && (o->n2 == 0 || (o->ba2_t && o->tri2 && o->mirror2));
}

}  // namespace

int launch_gsis_hot_apply(pbte_ctx *c, const pbte_gsis_ops *o, const double *vdf, double tc5, double *aa_src,
                          cudaStream_t s) {
    if (!ops_ok(o) || o->n_tris != c->n_tris || o->ndof != c->nd) return PBTE_ERR_ARG;
    const int total = c->n_tris * c->nd;
    const size_t shm = (size_t)4 * c->ndir * sizeof(double);
    if (shm > 48 * 1024) {
        if (shm > 200 * 1024) return PBTE_ERR_UNSUPPORTED;
        if (cudaFuncSetAttribute(hot_moments_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm) !=
            cudaSuccess)
            return PBTE_ERR_CUDA;
    }
    hot_moments_kernel<<<(total + kLanes - 1) / kLanes, dim3(kLanes, kChunks), shm, s>>>(
        vdf, c->d_cx, c->d_cy, c->d_w, c->ndir, total, c->d_gsis, c->done);
    const int M = 7 * c->nd;
    int th = 0;
    const int bl = elements_grid(c->n_tris, M, &th);
    const size_t hshm = (size_t)(th / M) * 4 * c->nd * sizeof(double);
    hot_apply_kernel<<<bl, th, hshm, s>>>(c->d_gsis, c->d_cells64, c->d_ref64, c->n_tris, c->nd, tc5, o->inv_t,
                                          aa_src, c->done);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// The FP32 GSIS product of the mixed-precision GSIS solve (its inner
// operator, whose accuracy the FP64 defect correction around it sets): the
// same steps on the folded FP32 distribution (one row per distinct in-plane
// velocity u; z-mirror twins are equal, so a pair's weights are summed: the
// d_u*64 arrays), FP32 products and sums, FP64 outputs.
namespace {

__global__ void __launch_bounds__(kLanes *kChunks) hot_moments32_kernel(const float *vdf, const double *cx,
                                                                        const double *cy, const double *w, int nu,
                                                                        int total, double *mk, const int32_t *done) {
    if (stopped(done)) return;
    extern __shared__ float ws32[];   // [4][nu]
    const int tid = threadIdx.y * kLanes + threadIdx.x;
    for (int u = tid; u < nu; u += kLanes * kChunks) {
        double a[4];
        weights<true>(cx[u], cy[u], w[u], a);
#pragma unroll
        for (int k = 0; k < 4; ++k) ws32[k * nu + u] = (float)a[k];
    }
    __syncthreads();
    const int t = blockIdx.x * kLanes + threadIdx.x;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    if (t < total)
        for (int u = threadIdx.y; u < nu; u += kChunks) {
            const float f = vdf[(size_t)u * total + t];
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[k] += ws32[k * nu + u] * f;
        }
    double accd[4] = {acc[0], acc[1], acc[2], acc[3]};
    reduce_chunks(accd, 4);
    if (threadIdx.y == 0 && t < total)
#pragma unroll
        for (int k = 0; k < 4; ++k) mk[(size_t)k * total + t] = accd[k];
}

__global__ void __launch_bounds__(kTraceThreads) wall_trace32_kernel(const float *vdf, const double *tri_fc_fc,
                                                                     const double *cx, const double *cy,
                                                                     const double *w, int nu, int nt, int NP, int NF,
                                                                     const int32_t *tri_list, const int32_t *lfc_list,
                                                                     double *out, const int32_t *done) {
    if (stopped(done)) return;
    __shared__ float c[16 * kMaxNf];
    __shared__ float red[3 * kMaxNf][kTraceThreads];
    const int k = blockIdx.x;
    const int tri = tri_list[k], lfc = lfc_list[k];
    for (int e = threadIdx.x; e < NP * NF; e += blockDim.x) {
        const int l = e / NF, m = e % NF;
        c[e] = (float)tri_fc_fc[(((size_t)l * NF + m) * nt + tri) * 3 + lfc];
    }
    __syncthreads();
    float acc[3 * kMaxNf];
    for (int q = 0; q < 3 * NF; ++q) acc[q] = 0.f;
    for (int u = threadIdx.x; u < nu; u += blockDim.x) {
        const float *f = vdf + ((size_t)u * nt + tri) * NP;
        const float wu = (float)w[u], cxu = (float)cx[u], cyu = (float)cy[u];
        for (int m = 0; m < NF; ++m) {
            float tt = 0.f;
            for (int l = 0; l < NP; ++l) tt += f[l] * c[l * NF + m];
            acc[m] += tt * wu;
            acc[NF + m] += cxu * tt * wu;
            acc[2 * NF + m] += cyu * tt * wu;
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

// the correction's coefficients and new moments (correct_moments_kernel's
// arithmetic after FP32 angular sums); ts/qxs/qys may be null
__global__ void __launch_bounds__(kLanes *kChunks) correct_coef32_kernel(
    const float *vdf, const double *uq, const double *cx, const double *cy, const double *w, const double *tri_hmin,
    int nu, int nt, int NP, double cv, double tau_r, double tau_thr, int use_hmin, double *coef, double *ts,
    double *qxs, double *qys, const int32_t *done) {
    if (stopped(done)) return;
    const int total = nt * NP;
    const int t = blockIdx.x * kLanes + threadIdx.x;
    float acc[3] = {0.f, 0.f, 0.f};
    if (t < total)
        for (int u = threadIdx.y; u < nu; u += kChunks) {
            const float f = vdf[(size_t)u * total + t];
            const float fw = f * (float)w[u];
            acc[0] += fw;
            acc[1] += (float)cx[u] * fw;
            acc[2] += (float)cy[u] * fw;
        }
    double accd[4] = {acc[0], acc[1], acc[2], 0.0};
    reduce_chunks(accd, 3);
    if (threadIdx.y != 0 || t >= total) return;
    const int i = t / NP, m = t % NP;
    const double tau_loc = use_hmin ? tau_r / tri_hmin[i] : tau_r;
    const double beta = fmin(tau_loc, tau_thr) / tau_loc;
    const double tv = accd[0] / cv, qxv = accd[1], qyv = accd[2];
    const double lt = (uq[(size_t)m * nt + i] - tv) * beta;
    const double lqx = (uq[(size_t)(NP + m) * nt + i] - qxv) * beta;
    const double lqy = (uq[(size_t)(2 * NP + m) * nt + i] - qyv) * beta;
    coef[t] = lt * cv / 4.0 / kPi;
    coef[total + t] = lqx;
    coef[2 * total + t] = lqy;
    if (ts) {
        ts[(size_t)m * nt + i] = lt + tv;
        qxs[(size_t)m * nt + i] = lqx + qxv;
        qys[(size_t)m * nt + i] = lqy + qyv;
    }
}

__global__ void correct_update32_kernel(float *vdf, const double *coef, const double *cx, const double *cy, int nu,
                                        int total, double drift, const int32_t *done) {
    if (stopped(done)) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const float eq = (float)coef[t], lqx = (float)(coef[total + t] * drift), lqy = (float)(coef[2 * total + t] * drift);
    for (int u = blockIdx.y; u < nu; u += gridDim.y) {
        float *f = vdf + (size_t)u * total + t;
        *f = *f + eq + ((float)cx[u] * lqx + (float)cy[u] * lqy);
    }
}

}  // namespace

int launch_gsis_product32(pbte_ctx *c, const pbte_gsis_ops *o, int step, float *vdf32, double tc5,
                          const double *tri_fc_fc, int nk, const int32_t *tri_list, const int32_t *lfc_list,
                          double *aa_src_or_wall, const double *uq, const double *tri_hmin, double tau_thr,
                          int use_hmin, double *const *mom_out, cudaStream_t s) {
    const int total = c->n_tris * c->nd;
    const int nu = c->n_udir;
    if (step == 0) {   // hot source with the element inverses -> aa_src
        if (!ops_ok(o) || o->n_tris != c->n_tris || o->ndof != c->nd) return PBTE_ERR_ARG;
        const size_t shm = (size_t)4 * nu * sizeof(float);
        if (shm > 48 * 1024) {
            if (shm > 200 * 1024) return PBTE_ERR_UNSUPPORTED;
            if (cudaFuncSetAttribute(hot_moments32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm) !=
                cudaSuccess)
                return PBTE_ERR_CUDA;
        }
        hot_moments32_kernel<<<(total + kLanes - 1) / kLanes, dim3(kLanes, kChunks), shm, s>>>(
            vdf32, c->d_ucx64, c->d_ucy64, c->d_uw64, nu, total, c->d_gsis, c->done);
        const int M = 7 * c->nd;
        int th = 0;
        const int bl = elements_grid(c->n_tris, M, &th);
        const size_t hshm = (size_t)(th / M) * 4 * c->nd * sizeof(double);
        hot_apply_kernel<<<bl, th, hshm, s>>>(c->d_gsis, c->d_cells64, c->d_ref64, c->n_tris, c->nd, tc5, o->inv_t,
                                              aa_src_or_wall, c->done);
    } else if (step == 1) {   // kinetic wall traces -> wall moments
        if (nk <= 0) return PBTE_OK;
        if (c->nd > 16 || c->nf > kMaxNf) return PBTE_ERR_UNSUPPORTED;
        wall_trace32_kernel<<<nk, kTraceThreads, 0, s>>>(vdf32, tri_fc_fc, c->d_ucx64, c->d_ucy64, c->d_uw64, nu,
                                                         c->n_tris, c->nd, c->nf, tri_list, lfc_list, aa_src_or_wall,
                                                         c->done);
    } else {   // the damped correction of the distribution
        correct_coef32_kernel<<<(total + kLanes - 1) / kLanes, dim3(kLanes, kChunks), 0, s>>>(
            vdf32, uq, c->d_ucx64, c->d_ucy64, c->d_uw64, tri_hmin, nu, c->n_tris, c->nd, c->cv, c->tau_r, tau_thr,
            use_hmin, c->d_gsis, mom_out ? mom_out[0] : nullptr, mom_out ? mom_out[1] : nullptr,
            mom_out ? mom_out[2] : nullptr, c->done);
        const double drift = c->tau_c / c->tau_n * 3.0 / 4.0 / kPi / c->vg / c->vg;
        const int th = 256;
        correct_update32_kernel<<<dim3((total + th - 1) / th, std::min(nu, 16)), th, 0, s>>>(
            vdf32, c->d_gsis, c->d_ucx64, c->d_ucy64, nu, total, drift, c->done);
    }
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

}  // namespace pbte

extern "C" int pbte_gsis_hot_apply(pbte_ctx *c, const pbte_gsis_ops *o, const double *vdf, double tc5,
                                   double *aa_src, void *stream) {
    if (!c || !vdf || !aa_src) return PBTE_ERR_ARG;
    return pbte::launch_gsis_hot_apply(c, o, vdf, tc5, aa_src, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int pbte_gsis_apply_inverse(const pbte_gsis_ops *o, const double *work, int32_t c0, int32_t c1,
                                       double *aa_src, const int32_t *done, void *stream) {
    if (!pbte::ops_ok(o) || !work || !aa_src || c0 < 0 || c1 > 7 * o->ndof || c0 > c1) return PBTE_ERR_ARG;
    int th = 0;
    const int bl = pbte::elements_grid(o->n_tris, 7 * o->ndof, &th);
    pbte::apply_inverse_kernel<<<bl, th, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        o->n_tris, 7 * o->ndof, o->inv_t, work, c0, c1, aa_src, done);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

extern "C" int pbte_gsis_trace_rhs(const pbte_gsis_ops *o, const double *aa_src, const double *wall_mom,
                                   double *ffa, const int32_t *done, void *stream) {
    if (!pbte::ops_ok(o) || !aa_src || !ffa) return PBTE_ERR_ARG;
    if (o->n_walls > 0 && (!wall_mom || !o->wall_nx || !o->wall_ny)) return PBTE_ERR_ARG;
    const long long total = (long long)o->n_faces * 3 * o->ndof_fc;
    const int th = 256;
    pbte::trace_rhs_kernel<<<(unsigned)((total + th - 1) / th), th, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        *o, aa_src, wall_mom, ffa, done);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

extern "C" int pbte_gsis_local_recover(const pbte_gsis_ops *o, const double *aa_src, const double *u_trace,
                                       double *uq, const int32_t *done, void *stream) {
    if (!pbte::ops_ok(o) || !aa_src || !u_trace || !uq) return PBTE_ERR_ARG;
    int th = 0;
    const int bl = pbte::elements_grid(o->n_tris, 7 * o->ndof, &th);
    pbte::local_recover_kernel<<<bl, th, 0, reinterpret_cast<cudaStream_t>(stream)>>>(*o, aa_src, u_trace, uq,
                                                                                      done);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

// ---- the FP32 GSIS product of the mixed-precision GSIS solve ---------------
static bool fold_ok(pbte_ctx *c) { return c && !c->has_periodic && (c->nd == 3 || c->nd == 6 || c->nd == 10); }

extern "C" int pbte_sweep_fold_f32(pbte_ctx *c, const double *ts, const double *qxs, const double *qys,
                                   const double *flux_wall, double wall_scale, float *vdf32, void *stream) {
    if (!fold_ok(c)) return c ? PBTE_ERR_UNSUPPORTED : PBTE_ERR_ARG;
    if (!ts || !qxs || !qys || !vdf32 || (c->n_wall_ad && !flux_wall)) return PBTE_ERR_ARG;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int rc = pbte::launch_sources(c, ts, qxs, qys, true, s);
    if (rc == PBTE_OK) rc = pbte::launch_sweep32(c, vdf32, flux_wall, wall_scale, s, false, true);
    return rc;
}

extern "C" int pbte_fold_epilogue_f32(pbte_ctx *c, const float *vdf32, double *ts, double *qxs, double *qys,
                                      double *flux_wall, double *temp, double *qx, double *qy, void *stream) {
    if (!fold_ok(c)) return c ? PBTE_ERR_UNSUPPORTED : PBTE_ERR_ARG;
    if (!vdf32 || !ts || !qxs || !qys) return PBTE_ERR_ARG;
    if ((temp == nullptr) != (qx == nullptr) || (temp == nullptr) != (qy == nullptr)) return PBTE_ERR_ARG;
    return pbte::launch_fold_epilogue32(c, vdf32, ts, qxs, qys, flux_wall, temp, qx, qy,
                                        reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int pbte_gsis_hot_apply_f32(pbte_ctx *c, const pbte_gsis_ops *o, const float *vdf32, double tc5,
                                       double *aa_src, void *stream) {
    if (!fold_ok(c)) return c ? PBTE_ERR_UNSUPPORTED : PBTE_ERR_ARG;
    if (!vdf32 || !aa_src) return PBTE_ERR_ARG;
    return pbte::launch_gsis_product32(c, o, 0, const_cast<float *>(vdf32), tc5, nullptr, 0, nullptr, nullptr,
                                       aa_src, nullptr, nullptr, 0.0, 0, nullptr,
                                       reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int pbte_wall_trace_f32(pbte_ctx *c, const float *vdf32, const double *tri_fc_fc, int32_t nk,
                                   const int32_t *tri_list, const int32_t *lfc_list, double *out, void *stream) {
    if (!fold_ok(c)) return c ? PBTE_ERR_UNSUPPORTED : PBTE_ERR_ARG;
    if (!vdf32 || nk < 0 || (nk && (!tri_fc_fc || !tri_list || !lfc_list || !out))) return PBTE_ERR_ARG;
    return pbte::launch_gsis_product32(c, nullptr, 1, const_cast<float *>(vdf32), 0.0, tri_fc_fc, nk, tri_list,
                                       lfc_list, out, nullptr, nullptr, 0.0, 0, nullptr,
                                       reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int pbte_correct_f32(pbte_ctx *c, float *vdf32, const double *uq, const double *tri_hmin,
                                double tau_thr, int use_hmin, double *ts, double *qxs, double *qys, void *stream) {
    if (!fold_ok(c)) return c ? PBTE_ERR_UNSUPPORTED : PBTE_ERR_ARG;
    if (!vdf32 || !uq || !tri_hmin) return PBTE_ERR_ARG;
    if ((ts == nullptr) != (qxs == nullptr) || (ts == nullptr) != (qys == nullptr)) return PBTE_ERR_ARG;
    double *const mom[3] = {ts, qxs, qys};
    return pbte::launch_gsis_product32(c, nullptr, 2, vdf32, 0.0, nullptr, 0, nullptr, nullptr, nullptr, uq,
                                       tri_hmin, tau_thr, use_hmin, ts ? mom : nullptr,
                                       reinterpret_cast<cudaStream_t>(stream));
}
