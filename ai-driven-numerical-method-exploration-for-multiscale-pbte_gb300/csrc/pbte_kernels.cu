// Device kernels of libpbte_gb300 (sm_103a).
//
// Transport sweep (pybte/_kernels.py:107-269).  One thread block walks one
// ordinate's wavefront levels; the threads of the block split the elements
// of a level, and each thread forms its element's N_p x N_p operator
//     A = area2 [ M/tau_c - (c.grad-xi) Dx - (c.grad-eta) Dy ] + sum_out (c.n) L_e R_e
// from the six reference matrices in shared memory, adds the upwind inflow
// through the edge gather map, and solves A x = b with partial pivoting in
// registers (or with stored FP64 factors in the "precomputed" mode).
// Other kernels: moment sources, moments, adiabatic-wall emission, residuals,
// transport residual, batched inverse (the GSIS kernels on the distribution
// are in pbte_gsis.cu).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "pbte_device.cuh"

namespace pbte {

template <typename T, int DEG, bool PRECOMP>
__global__ void __launch_bounds__(kSweepThreads) sweep_kernel(SweepParams<T> P) {
    constexpr int NP = Shape<DEG>::NP;
    __shared__ T sref[6 * NP * NP];
    if (stopped(P.done)) return;
    const int d = blockIdx.x;
    for (int k = threadIdx.x; k < 6 * NP * NP; k += blockDim.x) sref[k] = P.ref[k];
    __syncthreads();
    const T cx = (T)P.cx[d], cy = (T)P.cy[d];
    const int cls = P.dir_class[d];
    const int off = P.class_off[cls], nlev = P.class_nlev[cls];
    T *f = P.vdf + (size_t)d * P.nt * NP;
    int sing = 0;
    for (int L = 0; L < nlev; ++L) {
        const int beg = P.lvl_ptr[off + L], end = P.lvl_ptr[off + L + 1];
        for (int k = beg + threadIdx.x; k < end; k += blockDim.x) {
            const int i = P.lvl_cells[k];
            const CellRec<T> r = P.cells[i];
            T s[3];
#pragma unroll
            for (int il = 0; il < 3; ++il) s[il] = cx * r.nx[il] + cy * r.ny[il];
            T b[NP];
            rhs<T, DEG>(P, sref, r, i, d, cx, cy, s, f, b, P.fresh ? P.fresh[(size_t)cls * P.nt + i] : 0u);
            if constexpr (PRECOMP) {
                const int u = P.udir_of[d], p = k - cls * P.nt;
                const double *lu = P.lu + factor_base(u, p, P.nt, NP * NP);
                const int8_t *pv = P.piv + factor_base(u, p, P.nt, NP);
#pragma unroll
                for (int k2 = 0; k2 < NP; ++k2) {
                    const int pr = pv[32 * k2];
#pragma unroll
                    for (int j = k2 + 1; j < NP; ++j)
                        if (pr == j) { const T t = b[k2]; b[k2] = b[j]; b[j] = t; }
                }
#pragma unroll
                for (int k2 = 0; k2 < NP; ++k2)
#pragma unroll
                    for (int j = k2 + 1; j < NP; ++j) b[j] -= b[k2] * (T)lu[32 * (j * NP + k2)];
#pragma unroll
                for (int k2 = NP - 1; k2 >= 0; --k2) {
                    b[k2] *= (T)lu[32 * (k2 * NP + k2)];  // stored as 1/U_kk
#pragma unroll
                    for (int j = 0; j < k2; ++j) b[j] -= b[k2] * (T)lu[32 * (j * NP + k2)];
                }
            } else {
                T A[NP][NP];
                assemble<T, DEG>(sref, r, cx, cy, P.inv_tau_c, s, A);
                sing += lu_solve<T, NP>(A, b);
            }
            T *out = f + (size_t)i * NP;
#pragma unroll
            for (int m = 0; m < NP; ++m) out[m] = b[m];
        }
        __syncthreads();
    }
    if (sing) atomicAdd(P.singular, sing);
}

// Stored factors for the precomputed FP64 mode: LU with the row interchanges
// of partial pivoting, unit-lower multipliers below the diagonal, U above it
// and 1/U_kk on it; ipiv as in DGETF2.  One thread per (distinct in-plane
// velocity, sweep position), written in the factor_base() layout.
template <int DEG>
__global__ void factorise_kernel(SweepParams<double> P, double *lu_out, int8_t *piv_out,
                                 const int32_t *udir_rep, int n_udir) {
    constexpr int NP = Shape<DEG>::NP;
    __shared__ double sref[6 * NP * NP];
    for (int k = threadIdx.x; k < 6 * NP * NP; k += blockDim.x) sref[k] = P.ref[k];
    __syncthreads();
    const size_t total = (size_t)n_udir * P.nt;
    int sing = 0;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int u = (int)(t / P.nt), p = (int)(t % P.nt);
        const int d = udir_rep[u];
        const int i = P.lvl_cells[(size_t)P.dir_class[d] * P.nt + p];
        const double cx = P.cx[d], cy = P.cy[d];
        const CellRec<double> r = P.cells[i];
        double s[3];
        for (int il = 0; il < 3; ++il) s[il] = cx * r.nx[il] + cy * r.ny[il];
        double A[NP][NP];
        assemble<double, DEG>(sref, r, cx, cy, P.inv_tau_c, s, A);
        int8_t pv[NP];
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            double big = fabs(A[k][k]);
            int p = k;
#pragma unroll
            for (int i2 = k + 1; i2 < NP; ++i2) {
                const double v = fabs(A[i2][k]);
                if (v > big) { big = v; p = i2; }
            }
            pv[k] = (int8_t)p;
#pragma unroll
            for (int i2 = k + 1; i2 < NP; ++i2)
                if (p == i2)
#pragma unroll
                    for (int j = 0; j < NP; ++j) { const double tt = A[k][j]; A[k][j] = A[i2][j]; A[i2][j] = tt; }
            sing += (A[k][k] == 0.0);
            const double rr = 1.0 / A[k][k];
#pragma unroll
            for (int i2 = k + 1; i2 < NP; ++i2) {
                A[i2][k] *= rr;
#pragma unroll
                for (int j = k + 1; j < NP; ++j) A[i2][j] -= A[i2][k] * A[k][j];
            }
            A[k][k] = rr;
        }
        double *o = lu_out + factor_base(u, p, P.nt, NP * NP);
#pragma unroll
        for (int m = 0; m < NP; ++m)
#pragma unroll
            for (int l = 0; l < NP; ++l) o[32 * (m * NP + l)] = A[m][l];
        int8_t *po = piv_out + factor_base(u, p, P.nt, NP);
#pragma unroll
        for (int m = 0; m < NP; ++m) po[32 * m] = pv[m];
    }
    if (sing) atomicAdd(P.singular, sing);
}

// Moment sources: S[i][q][m] = area2_i sum_l M[l][m] mom_q[l][i], q = ts, qxs, qys.
template <typename T>
__global__ void sources_kernel(const CellRec<double> *cells, const double *ref_mass, const double *ts,
                               const double *qxs, const double *qys, T *S, int nt, int NP,
                               const int32_t *done) {
    if (stopped(done)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt) return;
    const double a2 = cells[i].area2;
    const double *mom[3] = {ts, qxs, qys};
    for (int q = 0; q < 3; ++q)
        for (int m = 0; m < NP; ++m) {
            double acc = 0.0;
            for (int l = 0; l < NP; ++l) acc += ref_mass[l * NP + m] * mom[q][(size_t)l * nt + i];
            S[((size_t)i * 3 + q) * NP + m] = (T)(a2 * acc);
        }
}

// Moments: one thread per (element, DOF); sum over ordinates in order.
template <typename T>
__global__ void moments_kernel(const T *vdf, const double *cx, const double *cy, const double *w, int ndir,
                               int nt, int NP, double cv, double *ts, double *qxs, double *qys,
                               const int32_t *done) {
    if (stopped(done)) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int total = nt * NP;
    if (t >= total) return;
    const int i = t / NP, l = t % NP;
    double ss = 0.0, ssx = 0.0, ssy = 0.0;
    if constexpr (sizeof(T) == 8) {
        for (int d = 0; d < ndir; ++d) {
            const double f = (double)vdf[(size_t)d * total + t];
            const double fw = f * w[d];
            ss += fw;
            ssx += cx[d] * fw;
            ssy += cy[d] * fw;
        }
    } else {
        // FP32 accumulation within blocks of 32 ordinates, FP64 across blocks
        for (int d0 = 0; d0 < ndir; d0 += 32) {
            float s0 = 0.f, sx = 0.f, sy = 0.f;
            const int d1 = min(ndir, d0 + 32);
            for (int d = d0; d < d1; ++d) {
                const float fw = (float)vdf[(size_t)d * total + t] * (float)w[d];
                s0 += fw;
                sx += (float)cx[d] * fw;
                sy += (float)cy[d] * fw;
            }
            ss += s0; ssx += sx; ssy += sy;
        }
    }
    ts[(size_t)l * nt + i] = ss / cv;
    qxs[(size_t)l * nt + i] = ssx;
    qys[(size_t)l * nt + i] = ssy;
}

// Moments in two passes: partial sums over chunks of kMomChunk ordinates
// (FP32 within a chunk for an FP32 distribution, FP64 otherwise), then a
// fixed-order FP64 sum of the chunks -- deterministic, and wide enough to fill
// the GPU (one thread per element DOF per chunk).
constexpr int kMomChunk = 32;

template <typename T>
__global__ void moments_partial_kernel(const T *vdf, const double *cx, const double *cy, const double *w,
                                       const float *cx32, const float *cy32, const float *w32,
                                       int ndir, int total, double *part, const int32_t *done) {
    if (stopped(done)) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int ch = blockIdx.y;
    if (t >= total) return;
    const int d0 = ch * kMomChunk, d1 = min(ndir, d0 + kMomChunk);
    double s0, sx, sy;
    if constexpr (sizeof(T) == 8) {
        s0 = sx = sy = 0.0;
        for (int d = d0; d < d1; ++d) {
            const double fw = vdf[(size_t)d * total + t] * w[d];
            s0 += fw;
            sx += cx[d] * fw;
            sy += cy[d] * fw;
        }
    } else {
        float a = 0.f, bx = 0.f, by = 0.f;
        for (int d = d0; d < d1; ++d) {
            const float fw = (float)vdf[(size_t)d * total + t] * w32[d];
            a += fw;
            bx += cx32[d] * fw;
            by += cy32[d] * fw;
        }
        s0 = a; sx = bx; sy = by;
    }
    double *p = part + (size_t)ch * 3 * total;
    p[t] = s0;
    p[total + t] = sx;
    p[2 * total + t] = sy;
}

__global__ void moments_combine_kernel(const double *part, int nch, int nt, int NP, double cv, double *ts,
                                       double *qxs, double *qys, const int32_t *done) {
    if (stopped(done)) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int total = nt * NP;
    if (t >= total) return;
    double s0 = 0.0, sx = 0.0, sy = 0.0;
    for (int ch = 0; ch < nch; ++ch) {
        const double *p = part + (size_t)ch * 3 * total;
        s0 += p[t];
        sx += p[total + t];
        sy += p[2 * total + t];
    }
    const int i = t / NP, l = t % NP;
    ts[(size_t)l * nt + i] = s0 / cv;
    qxs[(size_t)l * nt + i] = sx;
    qys[(size_t)l * nt + i] = sy;
}

__global__ void element_integrals_kernel(const double *ts, const double *qxs, const double *qys,
                                         const double *int_tri, int nt, int NP, double cv, double *temp,
                                         double *qx, double *qy, const int32_t *done) {
    if (stopped(done)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt) return;
    double a = 0.0, bx = 0.0, by = 0.0;
    for (int l = 0; l < NP; ++l) {
        const double it = int_tri[(size_t)l * nt + i];
        a += ts[(size_t)l * nt + i] * cv * it / cv;
        bx += qxs[(size_t)l * nt + i] * it;
        by += qys[(size_t)l * nt + i] * it;
    }
    temp[i] = a;
    qx[i] = bx;
    qy[i] = by;
}

// Block sum of the per-thread partial emissions (fixed tree) and the result
// -sum(u w f.fcm) / -sum(u w) of pybte/_kernels.py:385-397.
__device__ __forceinline__ void wall_flux_reduce(double *red, const double *acc, double s2, int NP, double *out) {
    for (int m = 0; m < NP; ++m) red[threadIdx.x * (NP + 1) + m] = acc[m];
    red[threadIdx.x * (NP + 1) + NP] = s2;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            for (int m = 0; m <= NP; ++m) red[threadIdx.x * (NP + 1) + m] += red[(threadIdx.x + h) * (NP + 1) + m];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double ss2 = red[NP];
        for (int m = 0; m < NP; ++m) out[m] = -red[m] / ss2;
    }
}

// Adiabatic-wall emission: one block per wall face, ordinates over threads.
template <typename T>
__global__ void wall_flux_kernel(const T *vdf, const WallFace *walls, const CellRec<double> *cells,
                                 const double *ref_edge, const double *cx, const double *cy,
                                 const double *w, int ndir, int nt, int NP, double *fw_out,
                                 const int32_t *done) {
    if (stopped(done)) return;
    extern __shared__ double red[];  // [blockDim][NP+1]
    const WallFace wf = walls[blockIdx.x];
    const double es = cells[wf.tri].es[wf.lfc];
    const double *R = ref_edge + (size_t)wf.lfc * NP * NP;
    double acc[16];
    for (int m = 0; m < NP; ++m) acc[m] = 0.0;
    double s2 = 0.0;
    for (int d = threadIdx.x; d < ndir; d += blockDim.x) {
        const double u = cx[d] * wf.nx + cy[d] * wf.ny;
        if (u < 0.0) {
            const T *f = vdf + ((size_t)d * nt + wf.tri) * NP;
            for (int m = 0; m < NP; ++m) {
                double a = 0.0;
                for (int l = 0; l < NP; ++l) a += (double)f[l] * (es * R[m * NP + l]);
                acc[m] += u * w[d] * a;
            }
        } else {
            s2 -= u * w[d];
        }
    }
    wall_flux_reduce(red, acc, s2, NP, fw_out + (size_t)wf.face * NP);
}

// The same with N_p known at compile time (registers, no local arrays) and
// the products in the distribution's precision; the sums stay FP64.
template <typename T, int NP>
__global__ void wall_flux_np_kernel(const T *vdf, const WallFace *walls, const CellRec<double> *cells,
                                    const T *ref_edge, const double *cx, const double *cy, const double *w,
                                    int ndir, int nt, double *fw_out, const int32_t *done) {
    if (stopped(done)) return;
    extern __shared__ double red[];  // [blockDim][NP+1]
    const WallFace wf = walls[blockIdx.x];
    const T es = (T)cells[wf.tri].es[wf.lfc];
    const T *R = ref_edge + (size_t)wf.lfc * NP * NP;
    double acc[16];
#pragma unroll
    for (int m = 0; m < NP; ++m) acc[m] = 0.0;
    double s2 = 0.0;
    for (int d = threadIdx.x; d < ndir; d += blockDim.x) {
        const double u = cx[d] * wf.nx + cy[d] * wf.ny;
        if (u < 0.0) {
            const T *f = vdf + ((size_t)d * nt + wf.tri) * NP;
            T fl[NP];
#pragma unroll
            for (int l = 0; l < NP; ++l) fl[l] = f[l];
            const double uw = u * w[d];
#pragma unroll
            for (int m = 0; m < NP; ++m) {
                T a = T(0);
#pragma unroll
                for (int l = 0; l < NP; ++l) a += fl[l] * (es * R[m * NP + l]);
                acc[m] += uw * (double)a;
            }
        } else {
            s2 -= u * w[d];
        }
    }
    wall_flux_reduce(red, acc, s2, NP, fw_out + (size_t)wf.face * NP);
}


// ---------------------------------------------------------------------------
// Folded FP32 forms for the fixed-point product of the mixed path: z-mirror
// twins see the same transport, so one row per distinct in-plane velocity u
// (ordinate rep[u]) is read with the pair's summed weight uw[u].
// ---------------------------------------------------------------------------

// The folded FP32 product's epilogue in one launch: blocks (tile, chunk) of
// 32 elements x NP DOFs take the moment sums of a chunk of kMomChunk distinct
// velocities; the last chunk block of a tile to finish (a per-tile ticket)
// adds the chunks in order and forms the tile's moments and element
// integrals, with moments_combine_kernel's and element_integrals_kernel's
// arithmetic.  Blocks past the tiles (chunk 0 only) take the adiabatic-wall
// emission: a warp per wall face, distinct velocities over lanes, FP32
// products, FP64 sums reduced by shuffles in a fixed order.
template <int NP>
__global__ void __launch_bounds__(32 * NP) fold_epilogue_kernel(
    const float *vdf, const float *ucx32, const float *ucy32, const float *uw32, int nu, int nt, double cv,
    double *part, uint32_t *tickets, double *ts, double *qxs, double *qys, const double *int_tri, double *temp,
    double *qx, double *qy, const WallFace *walls, int nwall, const CellRec<double> *cells, const float *ref_edge,
    const double *ucx, const double *ucy, const double *uw, double *fw_out, const int32_t *done) {
    if (stopped(done)) return;
    const int ntiles = (nt + 31) / 32;
    const int total = nt * NP;
    if ((int)blockIdx.x >= ntiles) {
        if (blockIdx.y != 0 || !fw_out) return;
        const int lane = threadIdx.x % 32;
        const int f = ((int)blockIdx.x - ntiles) * NP + threadIdx.x / 32;
        if (f >= nwall) return;
        const WallFace wf = walls[f];
        const float es = (float)cells[wf.tri].es[wf.lfc];
        const float *R = ref_edge + (size_t)wf.lfc * NP * NP;
        double acc[NP];
#pragma unroll
        for (int m = 0; m < NP; ++m) acc[m] = 0.0;
        double s2 = 0.0;
        for (int u = lane; u < nu; u += 32) {
            const double un = ucx[u] * wf.nx + ucy[u] * wf.ny;
            if (un < 0.0) {
                const float *fr = vdf + ((size_t)u * nt + wf.tri) * NP;
                float fl[NP];
#pragma unroll
                for (int l = 0; l < NP; ++l) fl[l] = fr[l];
                const double uwv = un * uw[u];
#pragma unroll
                for (int m = 0; m < NP; ++m) {
                    float a = 0.f;
#pragma unroll
                    for (int l = 0; l < NP; ++l) a += fl[l] * (es * R[m * NP + l]);
                    acc[m] += uwv * (double)a;
                }
            } else {
                s2 -= un * uw[u];
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int m = 0; m < NP; ++m) acc[m] += __shfl_xor_sync(0xffffffffu, acc[m], o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        }
        if (lane == 0) {
            double *out = fw_out + (size_t)wf.face * NP;
#pragma unroll
            for (int m = 0; m < NP; ++m) out[m] = -acc[m] / s2;
        }
        return;
    }
    __shared__ float sw[kMomChunk], sx[kMomChunk], sy[kMomChunk];
    __shared__ double mt[3][32 * NP];
    __shared__ bool last;
    const int ch = blockIdx.y, nch = gridDim.y;
    const int u0 = ch * kMomChunk, u1 = min(nu, u0 + kMomChunk);
    if ((int)threadIdx.x < u1 - u0) {
        sw[threadIdx.x] = uw32[u0 + threadIdx.x];
        sx[threadIdx.x] = ucx32[u0 + threadIdx.x];
        sy[threadIdx.x] = ucy32[u0 + threadIdx.x];
    }
    __syncthreads();
    const int t = blockIdx.x * 32 * NP + threadIdx.x;
    const bool live = t < total;
    if (live) {
        const float *f = vdf + (size_t)u0 * total + t;
        float a = 0.f, bx = 0.f, by = 0.f;
#pragma unroll 8
        for (int k = 0; k < u1 - u0; ++k) {
            const float fw = f[(size_t)k * total] * sw[k];
            a += fw;
            bx += sx[k] * fw;
            by += sy[k] * fw;
        }
        double *p = part + (size_t)ch * 3 * total;
        p[t] = a;
        p[total + t] = bx;
        p[2 * total + t] = by;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&tickets[blockIdx.x], 1u) == (unsigned)(nch - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (live) {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        for (int c = 0; c < nch; ++c) {
            const volatile double *p = part + (size_t)c * 3 * total;
            s0 += p[t];
            s1 += p[total + t];
            s2 += p[2 * total + t];
        }
        const int i = t / NP, l = t % NP;
        ts[(size_t)l * nt + i] = s0 / cv;
        qxs[(size_t)l * nt + i] = s1;
        qys[(size_t)l * nt + i] = s2;
        mt[0][threadIdx.x] = s0 / cv;
        mt[1][threadIdx.x] = s1;
        mt[2][threadIdx.x] = s2;
    }
    __syncthreads();
    if (threadIdx.x < 32 && temp) {
        const int i = blockIdx.x * 32 + threadIdx.x;
        if (i < nt) {
            double a = 0.0, bx = 0.0, by = 0.0;
#pragma unroll
            for (int l = 0; l < NP; ++l) {
                const double it = int_tri[(size_t)l * nt + i];
                a += mt[0][threadIdx.x * NP + l] * cv * it / cv;
                bx += mt[1][threadIdx.x * NP + l] * it;
                by += mt[2][threadIdx.x * NP + l] * it;
            }
            temp[i] = a;
            qx[i] = bx;
            qy[i] = by;
        }
    }
    if (threadIdx.x == 0) tickets[blockIdx.x] = 0u;
}

// Step residual and mass; out[0] = residual, out[1] = sum(temp); t_old <- temp.
__global__ void residual_kernel(const double *temp, double *t_old, int n, double *out, const int32_t *done) {
    if (stopped(done)) return;
    __shared__ double s1[1024], s2[1024], s3[1024];
    double a = 0.0, b = 0.0, c = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double d = temp[i] - t_old[i];
        a += d * d;
        b += temp[i] * temp[i];
        c += temp[i];
    }
    s1[threadIdx.x] = a; s2[threadIdx.x] = b; s3[threadIdx.x] = c;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            s1[threadIdx.x] += s1[threadIdx.x + h];
            s2[threadIdx.x] += s2[threadIdx.x + h];
            s3[threadIdx.x] += s3[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) { out[0] = sqrt(s1[0] / s2[0]); out[1] = s3[0]; }
    for (int i = threadIdx.x; i < n; i += blockDim.x) t_old[i] = temp[i];
}

// Convergence bookkeeping for graph-captured loops.  res[0] residual, res[1] mass;
// hist[2k], hist[2k+1] record them when hist is given.
__global__ void residual_check_kernel(const double *res, double tol, int64_t tmax, int32_t *done,
                                      int64_t *count, double *hist, int64_t hist_cap) {
    if (*done) return;
    const int64_t k = *count;
    if (hist && k < hist_cap) { hist[2 * k] = res[0]; hist[2 * k + 1] = res[1]; }
    *count = k + 1;
    if (res[0] < tol) *done = 1;
    else if (k + 1 >= tmax) *done = 2;
}

// ||A f - b||^2 per ordinate (no sweep): one block per ordinate.
template <int DEG>
__global__ void transport_residual_kernel(SweepParams<double> P, double *num, double *den) {
    constexpr int NP = Shape<DEG>::NP;
    __shared__ double sref[6 * NP * NP];
    __shared__ double r1[kSweepThreads], r2[kSweepThreads];
    const int d = blockIdx.x;
    for (int k = threadIdx.x; k < 6 * NP * NP; k += blockDim.x) sref[k] = P.ref[k];
    __syncthreads();
    const double cx = P.cx[d], cy = P.cy[d];
    const double *f = P.vdf + (size_t)d * P.nt * NP;
    double a = 0.0, b2 = 0.0;
    for (int i = threadIdx.x; i < P.nt; i += blockDim.x) {
        const CellRec<double> r = P.cells[i];
        double s[3];
        for (int il = 0; il < 3; ++il) s[il] = cx * r.nx[il] + cy * r.ny[il];
        double b[NP];
        // no sweep here: every periodic partner's current row is final
        rhs<double, DEG>(P, sref, r, i, d, cx, cy, s, f, b, 7u);
        double A[NP][NP];
        assemble<double, DEG>(sref, r, cx, cy, P.inv_tau_c, s, A);
        const double *fi = f + (size_t)i * NP;
#pragma unroll
        for (int m = 0; m < NP; ++m) {
            double rr = -b[m];
#pragma unroll
            for (int l = 0; l < NP; ++l) rr += A[m][l] * fi[l];
            a += rr * rr;
            b2 += b[m] * b[m];
        }
    }
    r1[threadIdx.x] = a;
    r2[threadIdx.x] = b2;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) { r1[threadIdx.x] += r1[threadIdx.x + h]; r2[threadIdx.x] += r2[threadIdx.x + h]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        num[d] = r1[0];
        den[d] = r2[0];
    }
}

__global__ void scale_by_weight_kernel(double *num, double *den, const double *w, int ndir) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d < ndir) { num[d] *= w[d]; den[d] *= w[d]; }
}

// Batched Gauss-Jordan inverse with partial pivoting, one warp per matrix,
// the augmented [A | I] rows held in shared memory.
__global__ void batched_inverse_kernel(const double *a, double *inv, int n, int m, int32_t *singular) {
    extern __shared__ double sm[];
    const int warps = blockDim.x / 32;
    const int wid = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int id = blockIdx.x * warps + wid;
    double *M = sm + (size_t)wid * m * 2 * m;
    if (id >= n) return;
    const int w2 = 2 * m;
    for (int k = lane; k < m * w2; k += 32) {
        const int r = k / w2, c = k % w2;
        M[k] = c < m ? a[(size_t)id * m * m + r * m + c] : (c - m == r ? 1.0 : 0.0);
    }
    __syncwarp();
    int sing = 0;
    for (int k = 0; k < m; ++k) {
        // pivot: first maximum |M[r][k]|, r >= k
        double best = -1.0;
        int p = k;
        for (int r = k + lane; r < m; r += 32) {
            const double v = fabs(M[r * w2 + k]);
            if (v > best) { best = v; p = r; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_down_sync(0xffffffffu, best, o);
            const int op = __shfl_down_sync(0xffffffffu, p, o);
            if (ob > best || (ob == best && op < p)) { best = ob; p = op; }
        }
        p = __shfl_sync(0xffffffffu, p, 0);
        if (p != k)
            for (int c = lane; c < w2; c += 32) {
                const double t = M[k * w2 + c]; M[k * w2 + c] = M[p * w2 + c]; M[p * w2 + c] = t;
            }
        __syncwarp();
        const double piv = M[k * w2 + k];
        if (piv == 0.0) { sing = 1; continue; }
        const double rp = 1.0 / piv;
        for (int c = lane; c < w2; c += 32) M[k * w2 + c] *= rp;
        __syncwarp();
        for (int r = 0; r < m; ++r) {
            if (r == k) continue;
            const double fct = M[r * w2 + k];
            __syncwarp();
            for (int c = lane; c < w2; c += 32) M[r * w2 + c] -= fct * M[k * w2 + c];
            __syncwarp();
        }
    }
    for (int k = lane; k < m * m; k += 32) inv[(size_t)id * m * m + k] = M[(k / m) * w2 + m + k % m];
    if (sing && lane == 0) atomicAdd(singular, 1);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <typename T>
static SweepParams<T> make_params(pbte_ctx *c) {
    SweepParams<T> P{};
    P.cx = c->d_cx; P.cy = c->d_cy;
    P.dir_class = c->d_dir_class; P.class_off = c->d_class_lvl_off; P.class_nlev = c->d_class_nlev;
    P.lvl_ptr = c->d_lvl_ptr; P.lvl_cells = c->d_lvl_cells;
    P.udir_of = c->d_udir_of;
    P.store_twin = 1;
    P.by_udir = 0;
    P.fresh = c->d_fresh;
    P.pslot = nullptr;
    P.pb_rows = c->n_faces;
    P.lu32 = c->d_lu32;
    P.singular = c->d_singular; P.done = c->done;
    P.nt = c->n_tris; P.n_faces = c->n_faces;
    P.inv_tau_c = (T)(1.0 / c->tau_c);
    P.ca = (T)(c->cv / (4.0 * kPi) * (1.0 / c->tau_r + 1.0 / c->tau_n));
    P.cb = (T)(3.0 / (4.0 * kPi) / (c->vg * c->vg) / c->tau_n);
    P.wall_scale = (T)1;
    return P;
}

// Moment sources with N_p at compile time, one thread per (element, moment).
template <typename T, int NP>
__global__ void sources_np_kernel(const CellRec<double> *cells, const double *ref_mass, const double *ts,
                                  const double *qxs, const double *qys, T *S, int nt, const int32_t *done) {
    if (stopped(done)) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * nt) return;
    const int i = t % nt, q = t / nt;
    const double *mom = q == 0 ? ts : (q == 1 ? qxs : qys);
    double v[NP];
#pragma unroll
    for (int l = 0; l < NP; ++l) v[l] = mom[(size_t)l * nt + i];
    const double a2 = cells[i].area2;
    T *o = S + ((size_t)i * 3 + q) * NP;
#pragma unroll
    for (int m = 0; m < NP; ++m) {
        double acc = 0.0;
#pragma unroll
        for (int l = 0; l < NP; ++l) acc += ref_mass[l * NP + m] * v[l];
        o[m] = (T)(a2 * acc);
    }
}

int launch_sources(pbte_ctx *c, const double *ts, const double *qxs, const double *qys, bool f32,
                   cudaStream_t s) {
    const int th = 128, bl = (c->n_tris + th - 1) / th;
    const int bl3 = (3 * c->n_tris + th - 1) / th;
    auto go = [&](auto k32, auto k64) {
        if (f32) k32<<<bl3, th, 0, s>>>(c->d_cells64, c->d_ref64, ts, qxs, qys, c->d_S32, c->n_tris, c->done);
        else k64<<<bl3, th, 0, s>>>(c->d_cells64, c->d_ref64, ts, qxs, qys, c->d_S64, c->n_tris, c->done);
        return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
    };
    switch (c->nd) {
        case 3: return go(sources_np_kernel<float, 3>, sources_np_kernel<double, 3>);
        case 6: return go(sources_np_kernel<float, 6>, sources_np_kernel<double, 6>);
        case 10: return go(sources_np_kernel<float, 10>, sources_np_kernel<double, 10>);
        default: break;
    }
    if (f32)
        sources_kernel<float><<<bl, th, 0, s>>>(c->d_cells64, c->d_ref64, ts, qxs, qys, c->d_S32, c->n_tris, c->nd, c->done);
    else
        sources_kernel<double><<<bl, th, 0, s>>>(c->d_cells64, c->d_ref64, ts, qxs, qys, c->d_S64, c->n_tris, c->nd, c->done);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

template <typename T, bool PRE>
static int sweep_dispatch(pbte_ctx *c, SweepParams<T> P, cudaStream_t s) {
    switch (c->deg) {
        case 1: sweep_kernel<T, 1, PRE><<<c->ndir, kSweepThreads, 0, s>>>(P); break;
        case 2: sweep_kernel<T, 2, PRE><<<c->ndir, kSweepThreads, 0, s>>>(P); break;
        case 3: sweep_kernel<T, 3, PRE><<<c->ndir, kSweepThreads, 0, s>>>(P); break;
        case 4: sweep_kernel<T, 4, PRE><<<c->ndir, kSweepThreads, 0, s>>>(P); break;
        default: return PBTE_ERR_UNSUPPORTED;
    }
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

// One thread per (ordinate, periodic face, DOF).  mode 0: the partner rows of
// vdf [ndir][nt][nd] into the compact [ndir][n_pfaces][nd]; mode 1: compact
// into the periodic-face rows of a full pbuf [ndir][n_faces][nd].
__global__ void periodic_copy_kernel(const double *src, double *dst, const int32_t *pface, const int32_t *ptri,
                                     int ndir, int npf, int nt, int nfaces, int nd, int mode, const int32_t *done) {
    if (stopped(done)) return;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = (size_t)ndir * npf * nd;
    if (t >= total) return;
    const int l = (int)(t % nd);
    const int q = (int)((t / nd) % npf);
    const int d = (int)(t / ((size_t)nd * npf));
    if (mode == 0) dst[t] = src[((size_t)d * nt + ptri[q]) * nd + l];
    else dst[((size_t)d * nfaces + pface[q]) * nd + l] = src[t];
}

int launch_periodic_copy(pbte_ctx *c, const double *src, double *dst, int mode, cudaStream_t s) {
    if (c->n_pfaces == 0) return PBTE_OK;
    const size_t total = (size_t)c->ndir * c->n_pfaces * c->nd;
    const int th = 256;
    periodic_copy_kernel<<<(unsigned)((total + th - 1) / th), th, 0, s>>>(
        src, dst, c->d_pface, c->d_ptri, c->ndir, c->n_pfaces, c->n_tris, c->n_faces, c->nd, mode, c->done);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

int launch_sweep64(pbte_ctx *c, double *vdf, const double *fw, const double *pbuf, int use_pbuf,
                   cudaStream_t s) {
    SweepParams<double> P = make_params<double>(c);
    P.cells = c->d_cells64; P.ref = c->d_ref64; P.S = c->d_S64; P.vdf = vdf;
    P.flux_wall = fw; P.pbuf = pbuf; P.use_pbuf = use_pbuf;
    P.lu = c->d_lu; P.piv = c->d_piv;
    if (c->has_periodic && !use_pbuf) {
        // source iteration: lagged partners read the values before this sweep
        const int rc = launch_periodic_copy(c, vdf, c->d_psnap, 0, s);
        if (rc) return rc;
        P.pbuf = c->d_psnap;
        P.pslot = c->d_pslot;
        P.pb_rows = c->n_pfaces;
    }
    if (c->sweep_variant != 1) {
        const int rc = c->d_lu ? launch_ring<double, true>(c, P, s) : launch_ring<double, false>(c, P, s);
        if (rc != PBTE_ERR_UNSUPPORTED || c->sweep_variant >= 2) return rc;
    }
    if (c->d_lu) return sweep_dispatch<double, true>(c, P, s);
    return sweep_dispatch<double, false>(c, P, s);
}

SweepParams<float> fold_params32(pbte_ctx *c, float *vdf32, const double *fw, double wall_scale,
                                 const int32_t *done) {
    SweepParams<float> P = make_params<float>(c);
    P.cells = c->d_cells32; P.ref = c->d_ref32; P.S = c->d_S32; P.vdf = vdf32;
    P.flux_wall = fw; P.wall_scale = (float)wall_scale;
    P.store_twin = 0;
    P.by_udir = 1;
    P.lu32 = nullptr;
    P.done = done;
    return P;
}

int launch_sweep32(pbte_ctx *c, float *vdf32, const double *fw, double wall_scale, cudaStream_t s,
                   bool store_twin, bool by_udir) {
    SweepParams<float> P = make_params<float>(c);
    P.cells = c->d_cells32; P.ref = c->d_ref32; P.S = c->d_S32; P.vdf = vdf32;
    P.flux_wall = fw; P.wall_scale = (float)wall_scale;
    P.store_twin = store_twin ? 1 : 0;
    P.by_udir = by_udir ? 1 : 0;
    if (by_udir) {
        // rows by distinct velocity exist only in the ring sweep
        if (c->sweep_variant == 1) return PBTE_ERR_UNSUPPORTED;
        return c->d_lu32 ? launch_ring<float, true>(c, P, s) : launch_ring<float, false>(c, P, s);
    }
    if (c->sweep_variant != 1) {
        const int rc = c->d_lu32 ? launch_ring<float, true>(c, P, s) : launch_ring<float, false>(c, P, s);
        if (rc != PBTE_ERR_UNSUPPORTED || c->sweep_variant >= 2) return rc;
    }
    return sweep_dispatch<float, false>(c, P, s);
}

int launch_factorise(pbte_ctx *c, cudaStream_t s) {
    SweepParams<double> P = make_params<double>(c);
    P.cells = c->d_cells64; P.ref = c->d_ref64;
    const int th = 128;
    const size_t total = (size_t)c->n_udir * c->n_tris;
    const int bl = (int)std::min<size_t>((total + th - 1) / th, 152 * 16);
    const int32_t *rep = c->d_udir_rep;
    switch (c->deg) {
        case 1: factorise_kernel<1><<<bl, th, 0, s>>>(P, c->d_lu, c->d_piv, rep, c->n_udir); break;
        case 2: factorise_kernel<2><<<bl, th, 0, s>>>(P, c->d_lu, c->d_piv, rep, c->n_udir); break;
        case 3: factorise_kernel<3><<<bl, th, 0, s>>>(P, c->d_lu, c->d_piv, rep, c->n_udir); break;
        case 4: factorise_kernel<4><<<bl, th, 0, s>>>(P, c->d_lu, c->d_piv, rep, c->n_udir); break;
        default: return PBTE_ERR_UNSUPPORTED;
    }
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

template <typename T>
static int moments_impl(pbte_ctx *c, const T *vdf, double *ts, double *qxs, double *qys, double *temp,
                        double *qx, double *qy, cudaStream_t s) {
    const int total = c->n_tris * c->nd, th = 256;
    const int nch = (c->ndir + kMomChunk - 1) / kMomChunk;
    if (c->d_mom_part) {
        moments_partial_kernel<T><<<dim3((total + th - 1) / th, nch), th, 0, s>>>(
            vdf, c->d_cx, c->d_cy, c->d_w, c->d_cx32, c->d_cy32, c->d_w32, c->ndir, total, c->d_mom_part, c->done);
        moments_combine_kernel<<<(total + th - 1) / th, th, 0, s>>>(c->d_mom_part, nch, c->n_tris, c->nd, c->cv, ts,
                                                                   qxs, qys, c->done);
    } else {
        moments_kernel<T><<<(total + th - 1) / th, th, 0, s>>>(vdf, c->d_cx, c->d_cy, c->d_w, c->ndir, c->n_tris,
                                                              c->nd, c->cv, ts, qxs, qys, c->done);
    }
    if (temp)
        element_integrals_kernel<<<(c->n_tris + th - 1) / th, th, 0, s>>>(ts, qxs, qys, c->d_int_tri, c->n_tris,
                                                                         c->nd, c->cv, temp, qx, qy, c->done);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

int launch_moments64(pbte_ctx *c, const double *vdf, double *ts, double *qxs, double *qys, double *temp,
                     double *qx, double *qy, cudaStream_t s) {
    return moments_impl<double>(c, vdf, ts, qxs, qys, temp, qx, qy, s);
}

int launch_moments32(pbte_ctx *c, const float *vdf, double *ts, double *qxs, double *qys, double *temp,
                     double *qx, double *qy, cudaStream_t s) {
    return moments_impl<float>(c, vdf, ts, qxs, qys, temp, qx, qy, s);
}

template <typename T>
static int wall_flux_impl(pbte_ctx *c, const T *vdf, double *fw, cudaStream_t s) {
    if (c->n_wall_ad == 0) return PBTE_OK;
    const int th = 64;
    const size_t shm = (size_t)th * (c->nd + 1) * sizeof(double);
    const T *ref_edge = nullptr;
    if constexpr (sizeof(T) == 8) ref_edge = c->d_ref64 + 3 * c->nd * c->nd;
    else ref_edge = c->d_ref32 + 3 * c->nd * c->nd;
    auto go = [&](auto kern) {
        kern<<<c->n_wall_ad, th, shm, s>>>(vdf, c->d_wall_ad, c->d_cells64, ref_edge, c->d_cx, c->d_cy, c->d_w,
                                           c->ndir, c->n_tris, fw, c->done);
    };
    switch (c->nd) {
        case 3: go(wall_flux_np_kernel<T, 3>); break;
        case 6: go(wall_flux_np_kernel<T, 6>); break;
        case 10: go(wall_flux_np_kernel<T, 10>); break;
        default:
            wall_flux_kernel<T><<<c->n_wall_ad, th, shm, s>>>(vdf, c->d_wall_ad, c->d_cells64,
                                                              c->d_ref64 + 3 * c->nd * c->nd, c->d_cx, c->d_cy,
                                                              c->d_w, c->ndir, c->n_tris, c->nd, fw, c->done);
    }
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

// q_{j+1} = w / h[j+1] as gmres_next_basis_kernel<float> does (row j+1 of
// the basis, widened into the operator input uin), one thread per state
// entry; a thread of the moment block (entry t = b * NP * nt + m * nt + e:
// moment b, DOF m, element e) also forms source entry (e, b, m) of the next
// sweep with sources_np_kernel's arithmetic, from the element's widened
// values of moment b (the other DOFs' entries are read again: they are in
// L1/L2).  Nothing once state[0] != 0.
template <int NP>
__global__ void next_basis_sources_kernel(int j, const float *__restrict__ w, const double *__restrict__ h,
                                          float *__restrict__ Q, long long ldq, double *__restrict__ uin,
                                          long long n, const int32_t *state, const CellRec<double> *cells,
                                          const double *__restrict__ ref_mass, float *__restrict__ S, int nt) {
    if (*(volatile const int32_t *)state != 0) return;
    const float hn = (float)h[j + 1];
    float *q = Q + (size_t)(j + 1) * ldq;
    const long long k = (long long)NP * nt;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const float f = w[t] / hn;
        q[t] = f;
        uin[t] = (double)f;
        if (t < 3 * k) {
            const int b = (int)(t / k);
            const long long r = t - b * k;
            const int m = (int)(r / nt), e = (int)(r - (long long)m * nt);
            const float *wb = w + b * k + e;
            double acc = 0.0;
#pragma unroll
            for (int l = 0; l < NP; ++l) acc += ref_mass[l * NP + m] * (double)(wb[(long long)l * nt] / hn);
            S[((size_t)e * 3 + b) * NP + m] = (float)(cells[e].area2 * acc);
        }
    }
}

int launch_next_basis_sources(pbte_ctx *c, int j, const float *w, const double *h, float *Q, int64_t ldq,
                              double *uin, int64_t n, const int32_t *state, cudaStream_t s) {
    const long long k = (long long)c->nd * c->n_tris;
    if (n < 3 * k || ldq < n) return PBTE_ERR_ARG;
    const int th = 256;
    const int bl = (int)std::min<long long>((n + th - 1) / th, 152 * 8);
    auto go = [&](auto kern) {
        kern<<<bl, th, 0, s>>>(j, w, h, Q, ldq, uin, n, state, c->d_cells64, c->d_ref64, c->d_S32, c->n_tris);
        return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
    };
    switch (c->nd) {
        case 3: return go(next_basis_sources_kernel<3>);
        case 6: return go(next_basis_sources_kernel<6>);
        case 10: return go(next_basis_sources_kernel<10>);
        default: return PBTE_ERR_UNSUPPORTED;
    }
}

int launch_fixed_point32(pbte_ctx *c, const double *ts, const double *qxs, const double *qys,
                         const double *fw_in, double wall_scale, float *vdf32, double *ts_out,
                         double *qxs_out, double *qys_out, double *fw_out, double *temp, double *qx,
                         double *qy, cudaStream_t s, bool with_sources) {
    // folded kernels exist for N_p = 3, 6, 10 and the ring sweep (which
    // writes rows by distinct velocity u); otherwise every ordinate is
    // stored and read
    bool fold = c->nd == 3 || c->nd == 6 || c->nd == 10;
    int rc = with_sources ? launch_sources(c, ts, qxs, qys, true, s) : PBTE_OK;
    if (rc) return rc;
    if (fold) {
        rc = launch_sweep32(c, vdf32, fw_in, wall_scale, s, false, true);
        if (rc == PBTE_ERR_UNSUPPORTED) fold = false;
        else if (rc) return rc;
    }
    if (!fold) {
        rc = launch_sweep32(c, vdf32, fw_in, wall_scale, s);
        if (rc == PBTE_OK) rc = moments_impl<float>(c, vdf32, ts_out, qxs_out, qys_out, temp, qx, qy, s);
        if (rc == PBTE_OK && fw_out) rc = wall_flux_impl<float>(c, vdf32, fw_out, s);
        return rc;
    }
    return launch_fold_epilogue32(c, vdf32, ts_out, qxs_out, qys_out, fw_out, temp, qx, qy, s);
}

// moments, element integrals and wall emission of a folded FP32 distribution
// (one row per distinct in-plane velocity) in one launch
int launch_fold_epilogue32(pbte_ctx *c, const float *vdf32, double *ts_out, double *qxs_out, double *qys_out,
                           double *fw_out, double *temp, double *qx, double *qy, cudaStream_t s) {
    if (!(c->nd == 3 || c->nd == 6 || c->nd == 10)) return PBTE_ERR_UNSUPPORTED;
    const int nch = (c->n_udir + kMomChunk - 1) / kMomChunk;
    const int ntiles = (c->n_tris + 31) / 32;
    const int nwall = fw_out ? c->n_wall_ad : 0;
    const float *ref_edge = c->d_ref32 + 3 * c->nd * c->nd;
    auto go = [&](auto kern, int np) {
        const int wall_blocks = (nwall + np - 1) / np;
        kern<<<dim3(ntiles + wall_blocks, nch), 32 * np, 0, s>>>(
            vdf32, c->d_ucx32, c->d_ucy32, c->d_uw32, c->n_udir, c->n_tris, c->cv, c->d_mom_part, c->d_tickets,
            ts_out, qxs_out, qys_out, c->d_int_tri, temp, qx, qy, c->d_wall_ad, nwall, c->d_cells64, ref_edge,
            c->d_ucx64, c->d_ucy64, c->d_uw64, fw_out, c->done);
    };
    switch (c->nd) {
        case 3: go(fold_epilogue_kernel<3>, 3); break;
        case 6: go(fold_epilogue_kernel<6>, 6); break;
        default: go(fold_epilogue_kernel<10>, 10); break;
    }
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

int launch_wall_flux64(pbte_ctx *c, const double *vdf, double *fw, cudaStream_t s) { return wall_flux_impl<double>(c, vdf, fw, s); }
int launch_wall_flux32(pbte_ctx *c, const float *vdf, double *fw, cudaStream_t s) { return wall_flux_impl<float>(c, vdf, fw, s); }

int launch_residual(pbte_ctx *c, const double *temp, double *t_old, double *out, cudaStream_t s) {
    residual_kernel<<<1, 1024, 0, s>>>(temp, t_old, c->n_tris, out, c->done);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

int launch_residual_check(pbte_ctx *c, const double *res, double tol, int64_t tmax, int32_t *done,
                          int64_t *count, double *hist, int64_t hist_cap, cudaStream_t s) {
    (void)c;
    residual_check_kernel<<<1, 1, 0, s>>>(res, tol, tmax, done, count, hist, hist_cap);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

int launch_transport_residual(pbte_ctx *c, const double *ts, const double *qxs, const double *qys,
                              const double *vdf, const double *fw, const double *pbuf, double *num,
                              double *den, cudaStream_t s) {
    int rc = launch_sources(c, ts, qxs, qys, false, s);
    if (rc) return rc;
    SweepParams<double> P = make_params<double>(c);
    P.done = nullptr;
    P.cells = c->d_cells64; P.ref = c->d_ref64; P.S = c->d_S64; P.vdf = const_cast<double *>(vdf);
    P.flux_wall = fw; P.pbuf = pbuf; P.use_pbuf = 0;
    switch (c->deg) {
        case 1: transport_residual_kernel<1><<<c->ndir, kSweepThreads, 0, s>>>(P, num, den); break;
        case 2: transport_residual_kernel<2><<<c->ndir, kSweepThreads, 0, s>>>(P, num, den); break;
        case 3: transport_residual_kernel<3><<<c->ndir, kSweepThreads, 0, s>>>(P, num, den); break;
        case 4: transport_residual_kernel<4><<<c->ndir, kSweepThreads, 0, s>>>(P, num, den); break;
        default: return PBTE_ERR_UNSUPPORTED;
    }
    scale_by_weight_kernel<<<(c->ndir + 127) / 128, 128, 0, s>>>(num, den, c->d_w, c->ndir);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

// The same two kernels with the moment sources in caller-provided device
// scratch of 3 * ndof * n_tris doubles instead of the context's own.
int launch_transport_residual_scratch(pbte_ctx *c, const double *ts, const double *qxs, const double *qys,
                                      const double *vdf, const double *fw, double *num, double *den,
                                      double *S, cudaStream_t s) {
    const int th = 128;
    sources_kernel<double><<<(c->n_tris + th - 1) / th, th, 0, s>>>(c->d_cells64, c->d_ref64, ts, qxs, qys, S,
                                                                   c->n_tris, c->nd, nullptr);
    SweepParams<double> P = make_params<double>(c);
    P.done = nullptr;
    P.cells = c->d_cells64; P.ref = c->d_ref64; P.S = S; P.vdf = const_cast<double *>(vdf);
    P.flux_wall = fw; P.pbuf = nullptr; P.use_pbuf = 0;
    switch (c->deg) {
        case 1: transport_residual_kernel<1><<<c->ndir, kSweepThreads, 0, s>>>(P, num, den); break;
        case 2: transport_residual_kernel<2><<<c->ndir, kSweepThreads, 0, s>>>(P, num, den); break;
        case 3: transport_residual_kernel<3><<<c->ndir, kSweepThreads, 0, s>>>(P, num, den); break;
        case 4: transport_residual_kernel<4><<<c->ndir, kSweepThreads, 0, s>>>(P, num, den); break;
        default: return PBTE_ERR_UNSUPPORTED;
    }
    scale_by_weight_kernel<<<(c->ndir + 127) / 128, 128, 0, s>>>(num, den, c->d_w, c->ndir);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

int launch_element_integrals(pbte_ctx *c, const double *ts, const double *qxs, const double *qys, double *temp,
                             double *qx, double *qy, cudaStream_t s) {
    const int th = 256;
    element_integrals_kernel<<<(c->n_tris + th - 1) / th, th, 0, s>>>(ts, qxs, qys, c->d_int_tri, c->n_tris, c->nd,
                                                                     c->cv, temp, qx, qy, nullptr);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

int launch_batched_inverse(const double *a, double *inv, int n, int m, int32_t *singular, cudaStream_t s) {
    if (n <= 0) return PBTE_OK;
    if (m <= 0) return PBTE_ERR_ARG;
    // one warp per matrix, its [m][2m] augmented copy in shared memory: up to
    // four warps a block while they fit (m = 7 N_p: 70 at P3, 105 at P4)
    const size_t per_warp = (size_t)m * 2 * m * sizeof(double);
    if (per_warp > 200 * 1024) return PBTE_ERR_UNSUPPORTED;
    const int warps = (int)std::max<size_t>(1, std::min<size_t>(4, (200 * 1024) / per_warp));
    const size_t shm = (size_t)warps * per_warp;
    if (shm > 48 * 1024 &&
        cudaFuncSetAttribute(batched_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm) != cudaSuccess)
        return PBTE_ERR_CUDA;
    batched_inverse_kernel<<<(n + warps - 1) / warps, warps * 32, shm, s>>>(a, inv, n, m, singular);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

}  // namespace pbte
