// Ring-pipelined transport sweep (the default sweep; pybte/_kernels.py:218-269).
//
// One thread block sweeps one distinct in-plane velocity (an ordinate and its
// z-mirror twin share it, so the block stores the result under both).  The
// block's threads form G groups of 64; group g owns the wavefront levels
// L = g, g+G, ...  For its level a group first does everything that does not
// depend on the upwind values -- read the element records (stored in the
// direction class's sweep order, so a level is one contiguous run), form the
// source and wall terms, assemble and LU-factor the element operators in
// registers (or load the stored FP64 factors), and fetch the records of its
// next level -- and only then waits for level L-1 (bar.sync on the barrier
// the previous group arrives at).  It then adds the upwind inflow from shared
// memory, finishes the two triangular solves, stores the result in shared
// memory, arrives on its own barrier for level L+1, and only after that
// writes the distribution to global memory.  The critical path per level is
// the inflow gather plus two small triangular solves; the factorisation of
// the next levels overlaps it on the other groups.
//
// Upwind values live in a near ring of the last R <= 4 levels (slot
// (level % R) * W + position) and, for the few dependencies that reach
// further back, in dedicated far slots; both are laid out on the host
// (pbte_ctx.cu) and referenced from the records.
#include <algorithm>

#include "pbte_device.cuh"

namespace pbte {

constexpr int kTPG = 64;        // threads per group
constexpr int kMaxGroups = 4;

struct RingParams {
    const void *recs;           // SweepRec<T>[nclass * n_tris] in sweep order
    const int32_t *class_W, *class_R;
    const int32_t *udir_rep, *udir_twin;
    int groups;
    int far_offset;             // start of the far slots, in values of T past the ring
};

__device__ __forceinline__ void bar_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void bar_arrive(int id, int n) { asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory"); }

template <typename T, int DEG, bool PRECOMP, int CPT>
__global__ void __launch_bounds__(kMaxGroups * kTPG) sweep_ring_kernel(SweepParams<T> P, RingParams Q) {
    constexpr int NP = Shape<DEG>::NP, NF = Shape<DEG>::NF;
    constexpr bool PF = (CPT == 1) && (sizeof(T) == 4);   // register prefetch of the next level's record
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sref = reinterpret_cast<T *>(smem_raw);
    T *ring = sref + 6 * NP * NP;
    T *far = ring + Q.far_offset;
    if (stopped(P.done)) return;
    const SweepRec<T> *recs = reinterpret_cast<const SweepRec<T> *>(Q.recs);
    const int u = blockIdx.x;
    const int d = Q.udir_rep[u], d2 = Q.udir_twin[u];
    for (int k = threadIdx.x; k < 6 * NP * NP; k += blockDim.x) sref[k] = P.ref[k];
    __syncthreads();
    const T cx = (T)P.cx[d], cy = (T)P.cy[d];
    const int cls = P.dir_class[d];
    const int off = P.class_off[cls], nlev = P.class_nlev[cls];
    const int W = Q.class_W[cls], Rr = Q.class_R[cls];
    const int G = Q.groups;
    const int g = threadIdx.x / kTPG, t = threadIdx.x % kTPG;
    T *f1 = P.vdf + (size_t)d * P.nt * NP;
    T *f2 = d2 >= 0 ? P.vdf + (size_t)d2 * P.nt * NP : nullptr;
    int sing = 0;
    SweepRec<T> nxt;
    if constexpr (PF) {
        if (g < nlev) {
            const int k = P.lvl_ptr[off + g] + t;
            if (k < P.lvl_ptr[off + g + 1]) nxt = recs[k];
        }
    }
    for (int L = g; L < nlev; L += G) {
        const int beg = P.lvl_ptr[off + L], end = P.lvl_ptr[off + L + 1];
        SweepRec<T> cur[CPT];
        bool valid[CPT];
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            const int k = beg + t + c * kTPG;
            valid[c] = k < end;
            if (valid[c]) {
                if constexpr (PF) cur[c] = nxt;
                else cur[c] = recs[k];
            }
        }
        T Sv[CPT][3 * NP];
#pragma unroll
        for (int c = 0; c < CPT; ++c)
            if (valid[c]) {
                const T *S = P.S + (size_t)cur[c].cell * 3 * NP;
#pragma unroll
                for (int q = 0; q < 3 * NP; ++q) Sv[c][q] = S[q];
            }
        if constexpr (PF) {
            const int Ln = L + G;
            if (Ln < nlev) {
                const int k = P.lvl_ptr[off + Ln] + t;
                if (k < P.lvl_ptr[off + Ln + 1]) nxt = recs[k];
            }
        }
        T A[CPT][NP][NP];
        T b[CPT][NP];
        int piv[CPT][NP];
        T scin[CPT][3];
        // ---- independent of the upwind values ------------------------------
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            if (!valid[c]) continue;
            const CellRec<T> &r = cur[c].c;
            const int i = cur[c].cell;
            T s[3];
#pragma unroll
            for (int il = 0; il < 3; ++il) {
                s[il] = cx * r.nx[il] + cy * r.ny[il];
                scin[c][il] = s[il] * r.es[il];
            }
            if constexpr (PRECOMP) {
                const double *lu = P.lu + ((size_t)d * P.nt + i) * NP * NP;
                const int8_t *pv = P.piv + ((size_t)d * P.nt + i) * NP;
#pragma unroll
                for (int m = 0; m < NP; ++m) {
                    piv[c][m] = pv[m];
#pragma unroll
                    for (int l = 0; l < NP; ++l) A[c][m][l] = (T)lu[m * NP + l];
                }
            } else if constexpr (sizeof(T) == 4) {
                // FP32: no row interchanges.  x^T A x = |x|^2_M / tau_c +
                // (1/2) sum_edges |c.n| |x|^2_edge > 0, so every leading block
                // is non-singular; the FP64 defect correction around the FP32
                // sweeps absorbs the extra rounding.
                assemble<T, DEG>(sref, r, cx, cy, P.inv_tau_c, s, A[c]);
#pragma unroll
                for (int kk = 0; kk < NP; ++kk) {
                    piv[c][kk] = kk;
                    sing += (A[c][kk][kk] == T(0));
                    const T rr = __frcp_rn(A[c][kk][kk]);
#pragma unroll
                    for (int ii = kk + 1; ii < NP; ++ii) {
                        A[c][ii][kk] *= rr;
#pragma unroll
                        for (int j = kk + 1; j < NP; ++j) A[c][ii][j] -= A[c][ii][kk] * A[c][kk][j];
                    }
                    A[c][kk][kk] = rr;
                }
            } else {
                assemble<T, DEG>(sref, r, cx, cy, P.inv_tau_c, s, A[c]);
                // partial pivoting (first maximum), multipliers below the
                // diagonal, 1/U_kk on it
#pragma unroll
                for (int kk = 0; kk < NP; ++kk) {
                    T big = fabs(A[c][kk][kk]);
                    int p = kk;
#pragma unroll
                    for (int ii = kk + 1; ii < NP; ++ii) {
                        const T v = fabs(A[c][ii][kk]);
                        if (v > big) { big = v; p = ii; }
                    }
                    piv[c][kk] = p;
#pragma unroll
                    for (int ii = kk + 1; ii < NP; ++ii)
                        if (p == ii)
#pragma unroll
                            for (int j = 0; j < NP; ++j) { const T tt = A[c][kk][j]; A[c][kk][j] = A[c][ii][j]; A[c][ii][j] = tt; }
                    sing += (A[c][kk][kk] == T(0));
                    const T rr = T(1) / A[c][kk][kk];
#pragma unroll
                    for (int ii = kk + 1; ii < NP; ++ii) {
                        A[c][ii][kk] *= rr;
#pragma unroll
                        for (int j = kk + 1; j < NP; ++j) A[c][ii][j] -= A[c][ii][kk] * A[c][kk][j];
                    }
                    A[c][kk][kk] = rr;
                }
            }
#pragma unroll
            for (int m = 0; m < NP; ++m) b[c][m] = P.ca * Sv[c][m] + P.cb * (cx * Sv[c][NP + m] + cy * Sv[c][2 * NP + m]);
#pragma unroll
            for (int il = 0; il < 3; ++il) {
                if (!(s[il] < T(0))) continue;
                const T *R = sref + (3 + il) * NP * NP;
                const int kind = r.kind[il];
                if (kind == 3) {
                    const double *pb = P.pbuf + ((size_t)d * P.n_faces + r.face[il]) * NP;
#pragma unroll
                    for (int a = 0; a < NF; ++a) {
                        const int ma = Shape<DEG>::edof(il, a);
                        T acc = T(0);
#pragma unroll
                        for (int bb = 0; bb < NF; ++bb) acc += R[ma * NP + Shape<DEG>::edof(il, bb)] * (T)pb[r.emap[il][bb]];
                        b[c][ma] -= scin[c][il] * acc;
                    }
                } else if (kind == 1) {
                    const T sc = s[il] * r.bval[il] * P.wall_scale * r.es[il];
#pragma unroll
                    for (int a = 0; a < NF; ++a) {
                        const int ma = Shape<DEG>::edof(il, a);
                        T rs = T(0);
#pragma unroll
                        for (int bb = 0; bb < NF; ++bb) rs += R[ma * NP + Shape<DEG>::edof(il, bb)];
                        b[c][ma] -= sc * rs;
                    }
                } else if (kind == 2) {
                    const double *fw = P.flux_wall + (size_t)r.face[il] * NP;
#pragma unroll
                    for (int m = 0; m < NP; ++m) b[c][m] -= s[il] * (-(T)fw[m]);
                }
            }
        }
        // ---- wait for level L-1, then the upwind inflow and the solves ------
        if (G > 1 && L > 0) bar_sync(1 + (L - 1) % G, 2 * kTPG);
        const int rbase = (L % Rr) * W;
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            if (!valid[c]) continue;
            const CellRec<T> &r = cur[c].c;
#pragma unroll
            for (int il = 0; il < 3; ++il) {
                const int code = cur[c].up[il];
                if (code == -1) continue;
                const T *up = code >= 0 ? ring + (size_t)code * NP : far + (size_t)(-code - 2) * NP;
                const T *R = sref + (3 + il) * NP * NP;
                T gv[NF];
#pragma unroll
                for (int bb = 0; bb < NF; ++bb) gv[bb] = up[r.emap[il][bb]];
#pragma unroll
                for (int a = 0; a < NF; ++a) {
                    const int ma = Shape<DEG>::edof(il, a);
                    T acc = T(0);
#pragma unroll
                    for (int bb = 0; bb < NF; ++bb) acc += R[ma * NP + Shape<DEG>::edof(il, bb)] * gv[bb];
                    b[c][ma] -= scin[c][il] * acc;
                }
            }
            if constexpr (sizeof(T) == 8) {
#pragma unroll
                for (int kk = 0; kk < NP; ++kk) {
                    const int p = piv[c][kk];
#pragma unroll
                    for (int j = kk + 1; j < NP; ++j)
                        if (p == j) { const T tt = b[c][kk]; b[c][kk] = b[c][j]; b[c][j] = tt; }
                }
            }
#pragma unroll
            for (int kk = 0; kk < NP; ++kk)
#pragma unroll
                for (int j = kk + 1; j < NP; ++j) b[c][j] -= b[c][kk] * A[c][j][kk];
#pragma unroll
            for (int kk = NP - 1; kk >= 0; --kk) {
                b[c][kk] *= A[c][kk][kk];
#pragma unroll
                for (int j = 0; j < kk; ++j) b[c][j] -= b[c][kk] * A[c][j][kk];
            }
            T *rs = ring + (size_t)(rbase + t + c * kTPG) * NP;
#pragma unroll
            for (int m = 0; m < NP; ++m) rs[m] = b[c][m];
            if (cur[c].far_out >= 0) {
                T *fs = far + (size_t)cur[c].far_out * NP;
#pragma unroll
                for (int m = 0; m < NP; ++m) fs[m] = b[c][m];
            }
        }
        if (G > 1) {
            if (L + 1 < nlev) bar_arrive(1 + L % G, 2 * kTPG);
        } else {
            __syncthreads();
        }
        // the distribution itself is not read back inside the sweep: store it
        // after the hand-over so the barrier does not wait on global stores
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            if (!valid[c]) continue;
            T *o1 = f1 + (size_t)cur[c].cell * NP;
#pragma unroll
            for (int m = 0; m < NP; ++m) o1[m] = b[c][m];
            if (f2) {
                T *o2 = f2 + (size_t)cur[c].cell * NP;
#pragma unroll
                for (int m = 0; m < NP; ++m) o2[m] = b[c][m];
            }
        }
    }
    if (sing) atomicAdd(P.singular, sing);
}

template <typename T, int DEG, bool PRE>
static int ring_launch_deg(pbte_ctx *c, const SweepParams<T> &P, const RingParams &Q, int cpt, size_t shm,
                           cudaStream_t s) {
    const int threads = Q.groups * kTPG;
    auto go = [&](auto kern) {
        if (shm > 48 * 1024 &&
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm) != cudaSuccess)
            return PBTE_ERR_CUDA;
        kern<<<c->n_udir, threads, shm, s>>>(P, Q);
        return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
    };
    switch (cpt) {
        case 1: return go(sweep_ring_kernel<T, DEG, PRE, 1>);
        case 2: return go(sweep_ring_kernel<T, DEG, PRE, 2>);
        case 4:
            if constexpr (sizeof(T) == 4 && DEG <= 2) return go(sweep_ring_kernel<T, DEG, PRE, 4>);
            return PBTE_ERR_UNSUPPORTED;
        default: return PBTE_ERR_UNSUPPORTED;
    }
}

// Returns PBTE_ERR_UNSUPPORTED when the ring form does not fit (the caller
// then uses the level-serial kernel).
template <typename T, bool PRE>
int launch_ring(pbte_ctx *c, const SweepParams<T> &P, cudaStream_t s) {
    if (c->deg > 3 || c->ring_W <= 0) return PBTE_ERR_UNSUPPORTED;
    int cpt = (c->ring_W + kTPG - 1) / kTPG;
    if (cpt == 3) cpt = 4;
    if (cpt > 4 || (cpt == 4 && (sizeof(T) != 4 || c->deg > 2)) || (c->deg == 3 && cpt > 1))
        return PBTE_ERR_UNSUPPORTED;
    const size_t ring_vals = (size_t)c->ring_R * c->ring_W * c->nd;
    const size_t shm = sizeof(T) * ((size_t)6 * c->nd * c->nd + ring_vals + (size_t)c->far_max * c->nd);
    if (shm > 200 * 1024) return PBTE_ERR_UNSUPPORTED;
    const int groups = c->ring_groups > 0 ? std::min(c->ring_groups, kMaxGroups) : kMaxGroups;
    const void *recs = sizeof(T) == 4 ? (const void *)c->d_srec32 : (const void *)c->d_srec64;
    RingParams Q{recs, c->d_class_W, c->d_class_R, c->d_udir_rep, c->d_udir_twin, groups, (int)ring_vals};
    switch (c->deg) {
        case 1: return ring_launch_deg<T, 1, PRE>(c, P, Q, cpt, shm, s);
        case 2: return ring_launch_deg<T, 2, PRE>(c, P, Q, cpt, shm, s);
        case 3: return ring_launch_deg<T, 3, PRE>(c, P, Q, cpt, shm, s);
        default: return PBTE_ERR_UNSUPPORTED;
    }
}

template int launch_ring<double, false>(pbte_ctx *, const SweepParams<double> &, cudaStream_t);
template int launch_ring<double, true>(pbte_ctx *, const SweepParams<double> &, cudaStream_t);
template int launch_ring<float, false>(pbte_ctx *, const SweepParams<float> &, cudaStream_t);

}  // namespace pbte
