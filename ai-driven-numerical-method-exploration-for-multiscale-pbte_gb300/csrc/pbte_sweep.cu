// Ring-pipelined transport sweep (the default sweep; pybte/_kernels.py:218-269).
//
// One thread block sweeps one distinct in-plane velocity (an ordinate and its
// z-mirror twin share it, so the block stores the result under both).  The
// block's threads form G groups of 64; group g owns the wavefront levels
// L = g, g+G, ...  For its level a group first does everything that does not
// depend on the upwind values -- read the element records, form the source
// and wall terms, assemble and LU-factor the element operators in registers
// (or load the stored FP64 factors) -- and only then waits for level L-1
// (bar.sync on the barrier the previous group arrives at).  It then adds the
// upwind inflow from shared memory, finishes the two triangular solves,
// stores the result in shared memory, arrives on its own barrier for level
// L+1, and only after that writes the distribution to global memory and
// prefetches the source rows of its next level into L1.  The critical path
// per level is the inflow gather plus two small triangular solves; the
// factorisation of the next levels overlaps it on the other groups.
//
// The records are field-major in the direction class's sweep order (a level
// is one contiguous run of positions), so each field read of a warp is one
// coalesced access: per-thread records (an array of structs) made the L1
// the busiest unit of the kernel and slowed the shared-memory traffic of the
// critical path queued behind it.  Only what the post-barrier part needs
// (upwind slot codes, packed edge maps, far slot, edge factors) is carried
// across the barrier in registers.
//
// Upwind values live in a near ring of the last R <= 4 levels (slot
// (level % R) * W + position) and, for the few dependencies that reach
// further back, in dedicated far slots; both are laid out on the host
// (pbte_ctx.cu) and referenced from the records.  The ring is safe for any G:
// level L+R overwrites level L's slot only after the barrier chain has
// passed L+R-1, and every level reads its inflow before it arrives.
#include <algorithm>
#include <type_traits>
#include <vector>

#include "pbte_internal.cuh"

#include "pbte_device.cuh"

namespace pbte {

constexpr int kMaxGroups = 8;

struct RingParams {
    const void *rf;             // T[kNumRecReal][stride]: real record fields in sweep order
    const int32_t *ri;          // [kNumRecInt][stride]: integer record fields
    int64_t stride;             // nclass * n_tris
    const int32_t *class_W, *class_R;
    const int32_t *udir_rep, *udir_twin;
    int groups;
    int far_offset;             // start of the far slots, in values of T past the ring
    int unfold;                 // one block per ordinate (no twin store): periodic faces
};

__device__ __forceinline__ void bar_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void bar_arrive(int id, int n) { asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void prefetch_l1(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// geometry of one element, as assemble() reads it
template <typename T>
struct Geo {
    T area2, gxa, gxb, gya, gyb, es[3];
};

// the element's three moment sources (3 * NP values, row i of P.S), in pairs
// where the row is 8-byte aligned for every i
template <typename T, int NP>
__device__ __forceinline__ void load_sources(const T *S, T (&v)[3 * NP]) {
    if constexpr (sizeof(T) == 4 && (3 * NP) % 2 == 0) {
        const float2 *s2 = reinterpret_cast<const float2 *>(S);
#pragma unroll
        for (int q = 0; q < 3 * NP / 2; ++q) {
            const float2 x = __ldg(s2 + q);
            v[2 * q] = x.x;
            v[2 * q + 1] = x.y;
        }
    } else {
#pragma unroll
        for (int q = 0; q < 3 * NP; ++q) v[q] = __ldg(S + q);
    }
}

// one element's NP values into its row of the distribution, in pairs where
// the row is 8-byte (float) or 16-byte (double) aligned for every element
template <typename T, int NP>
__device__ __forceinline__ void store_row(T *o, const T (&v)[NP]) {
    if constexpr (NP % 2 == 0) {
        using V2 = typename std::conditional<sizeof(T) == 4, float2, double2>::type;
        V2 *o2 = reinterpret_cast<V2 *>(o);
#pragma unroll
        for (int q = 0; q < NP / 2; ++q) {
            V2 x;
            x.x = v[2 * q];
            x.y = v[2 * q + 1];
            o2[q] = x;
        }
    } else {
#pragma unroll
        for (int q = 0; q < NP; ++q) o[q] = v[q];
    }
}

// TPG: threads per group; GMAX: the most groups the kernel is compiled for
// (its launch bound); CH: levels may be wider than TPG * CPT (run in chunks)
// The sweep of one velocity (block `bid` of the case's grid); the body of
// sweep_ring_kernel (one case) and sweep_ring_batch_kernel (many cases).
template <typename T, int DEG, bool PRECOMP, int CPT, int TPG, int GMAX, bool CH>
__device__ __forceinline__ void ring_body(const SweepParams<T> &P, const RingParams &Q, int bid,
                                          unsigned char *smem_raw) {
    constexpr int NP = Shape<DEG>::NP, NF = Shape<DEG>::NF;
    T *sref = reinterpret_cast<T *>(smem_raw);
    T *ring = sref + 6 * NP * NP;
    T *far = ring + Q.far_offset;
    if (stopped(P.done)) return;
    const T *__restrict__ rf = reinterpret_cast<const T *>(Q.rf);
    const int32_t *__restrict__ ri = Q.ri;
    const int64_t M = Q.stride;
    const int u = Q.unfold ? P.udir_of[bid] : bid;
    const int d = Q.unfold ? bid : Q.udir_rep[u];
    const int d2 = Q.unfold ? -1 : Q.udir_twin[u];
    for (int k = threadIdx.x; k < 6 * NP * NP; k += blockDim.x) sref[k] = P.ref[k];
    __syncthreads();
    const T cx = (T)P.cx[d], cy = (T)P.cy[d];
    const int cls = P.dir_class[d];
    const int off = P.class_off[cls], nlev = P.class_nlev[cls];
    const int W = Q.class_W[cls], Rr = Q.class_R[cls];
    const int G = Q.groups;
    const int g = threadIdx.x / TPG, t = threadIdx.x % TPG;
    T *f1 = P.vdf + (size_t)(P.by_udir ? u : d) * P.nt * NP;
    T *f2 = (d2 >= 0 && P.store_twin) ? P.vdf + (size_t)d2 * P.nt * NP : nullptr;
    int sing = 0;
    int beg = g < nlev ? P.lvl_ptr[off + g] : 0;
    int end = g < nlev ? P.lvl_ptr[off + g + 1] : 0;
    // element indices of this group's current level (read one level ahead, so
    // the source rows can be prefetched into L1 while the level before runs)
    int cell[CPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
        const int k = beg + t + c * TPG;
        cell[c] = k < end ? __ldg(ri + kICell * M + k) : 0;
    }
    for (int L = g; L < nlev; L += G) {
        const int Ln = L + G;
        const int nbeg = Ln < nlev ? P.lvl_ptr[off + Ln] : 0;
        const int nend = Ln < nlev ? P.lvl_ptr[off + Ln + 1] : 0;
        int ncell[CPT];
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            const int k = nbeg + t + c * TPG;
            ncell[c] = k < nend ? __ldg(ri + kICell * M + k) : -1;
        }
        const int rbase = (L % Rr) * W;
        // a level wider than the group's TPG * CPT cells runs in chunks of
        // that many; only the first waits for level L-1 and only the last
        // hands level L on, so registers do not grow with the level width
        for (int cb = beg; cb < end; cb += CPT * TPG) {
        const bool first = !CH || cb == beg, last = !CH || cb + CPT * TPG >= end;
        if (!first) {
#pragma unroll
            for (int c = 0; c < CPT; ++c) {
                const int k = cb + t + c * TPG;
                cell[c] = k < end ? __ldg(ri + kICell * M + k) : 0;
            }
        }
        bool valid[CPT];
#pragma unroll
        for (int c = 0; c < CPT; ++c) valid[c] = cb + t + c * TPG < end;
        T A[CPT][NP][NP];
        T b[CPT][NP];
        int piv[CPT][NP];
        T scin[CPT][3];
        int code[CPT][3];
        uint32_t emp[CPT][3];
        int fo[CPT];
        // ---- independent of the upwind values ------------------------------
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            if (!valid[c]) continue;
            const int64_t k = cb + t + c * TPG;
            const int i = cell[c];
            {
                // the source first, so its values are dead before the factorisation
                T Sv[3 * NP];
                load_sources<T, NP>(P.S + (size_t)i * 3 * NP, Sv);
#pragma unroll
                for (int m = 0; m < NP; ++m) b[c][m] = P.ca * Sv[m] + P.cb * (cx * Sv[NP + m] + cy * Sv[2 * NP + m]);
            }
            Geo<T> r;
            T s[3];
#pragma unroll
            for (int il = 0; il < 3; ++il) {
                r.es[il] = __ldg(rf + (kREs + il) * M + k);
                s[il] = cx * __ldg(rf + (kRNx + il) * M + k) + cy * __ldg(rf + (kRNy + il) * M + k);
                scin[c][il] = s[il] * r.es[il];
                code[c][il] = __ldg(ri + (kIUp + il) * M + k);
                emp[c][il] = (uint32_t)__ldg(ri + (kIEmp + il) * M + k);
            }
            fo[c] = __ldg(ri + kIFarOut * M + k);
            const uint32_t kinds = (uint32_t)__ldg(ri + kIKind * M + k);
#pragma unroll
            for (int il = 0; il < 3; ++il) {
                if (!(s[il] < T(0))) continue;
                const T *R = sref + (3 + il) * NP * NP;
                const int kind = (kinds >> (8 * il)) & 255u;
                if (kind == 0) continue;
                // a fresh periodic partner comes from the ring like an
                // interior neighbour, unless the inflow is explicit state
                if (kind == 4 && !P.use_pbuf) continue;
                if (kind == 4) code[c][il] = -1;
                const int face = __ldg(ri + (kIFace + il) * M + k);
                if (kind == 3 || kind == 4) {
                    const int row = P.pslot ? P.pslot[face] : face;
                    const double *pb = P.pbuf + ((size_t)d * P.pb_rows + row) * NP;
#pragma unroll
                    for (int a = 0; a < NF; ++a) {
                        const int ma = Shape<DEG>::edof(il, a);
                        T acc = T(0);
#pragma unroll
                        for (int bb = 0; bb < NF; ++bb)
                            acc += R[ma * NP + Shape<DEG>::edof(il, bb)] * (T)pb[(emp[c][il] >> (4 * bb)) & 15u];
                        b[c][ma] -= scin[c][il] * acc;
                    }
                } else if (kind == 1) {
                    const T sc = s[il] * __ldg(rf + (kRBval + il) * M + k) * P.wall_scale * r.es[il];
#pragma unroll
                    for (int a = 0; a < NF; ++a) {
                        const int ma = Shape<DEG>::edof(il, a);
                        T rs = T(0);
#pragma unroll
                        for (int bb = 0; bb < NF; ++bb) rs += R[ma * NP + Shape<DEG>::edof(il, bb)];
                        b[c][ma] -= sc * rs;
                    }
                } else if (kind == 2) {
                    const double *fw = P.flux_wall + (size_t)face * NP;
#pragma unroll
                    for (int m = 0; m < NP; ++m) b[c][m] -= s[il] * (-(T)fw[m]);
                }
            }
            if constexpr (!PRECOMP) {
                r.area2 = __ldg(rf + kRA2 * M + k);
                r.gxa = __ldg(rf + kRGxa * M + k);
                r.gxb = __ldg(rf + kRGxb * M + k);
                r.gya = __ldg(rf + kRGya * M + k);
                r.gyb = __ldg(rf + kRGyb * M + k);
            }
            if constexpr (PRECOMP && sizeof(T) == 4) {
                // stored FP32 factors (factorise32_kernel): no interchanges
                const int p = (int)(k - (int64_t)cls * P.nt);
                const float *lu = P.lu32 + factor_base(u, p, P.nt, NP * NP);
#pragma unroll
                for (int m = 0; m < NP; ++m) {
                    piv[c][m] = m;
#pragma unroll
                    for (int l = 0; l < NP; ++l) A[c][m][l] = __ldg(lu + 32 * (m * NP + l));
                }
            } else if constexpr (PRECOMP) {
                const int p = (int)(k - (int64_t)cls * P.nt);
                const double *lu = P.lu + factor_base(u, p, P.nt, NP * NP);
                const int8_t *pv = P.piv + factor_base(u, p, P.nt, NP);
#pragma unroll
                for (int m = 0; m < NP; ++m) {
                    piv[c][m] = __ldg(pv + 32 * m);
#pragma unroll
                    for (int l = 0; l < NP; ++l) A[c][m][l] = (T)__ldg(lu + 32 * (m * NP + l));
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
        }
        // ---- wait for level L-1, then the upwind inflow and the solves ------
        if (first && G > 1 && L > 0) bar_sync(1 + (L - 1) % G, 2 * TPG);
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            if (!valid[c]) continue;
#pragma unroll
            for (int il = 0; il < 3; ++il) {
                const int cd = code[c][il];
                if (cd == -1) continue;
                const T *up = cd >= 0 ? ring + (size_t)cd * NP : far + (size_t)(-cd - 2) * NP;
                const T *R = sref + (3 + il) * NP * NP;
                T gv[NF];
#pragma unroll
                for (int bb = 0; bb < NF; ++bb) gv[bb] = up[(emp[c][il] >> (4 * bb)) & 15u];
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
            T *rs = ring + (size_t)(rbase + (cb - beg) + t + c * TPG) * NP;
#pragma unroll
            for (int m = 0; m < NP; ++m) rs[m] = b[c][m];
            if (fo[c] >= 0) {
                T *fs = far + (size_t)fo[c] * NP;
#pragma unroll
                for (int m = 0; m < NP; ++m) fs[m] = b[c][m];
            }
        }
        if (last) {
            if (G > 1) {
                if (L + 1 < nlev) bar_arrive(1 + L % G, 2 * TPG);
            } else {
                __syncthreads();
            }
        }
        // the distribution itself is not read back inside the sweep: store it
        // after the hand-over so the barrier does not wait on global stores
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            if (!valid[c]) continue;
            store_row<T, NP>(f1 + (size_t)cell[c] * NP, b[c]);
            if (f2) store_row<T, NP>(f2 + (size_t)cell[c] * NP, b[c]);
        }
        if (!CH) break;
        }   // chunks of the level
        // the next level's source rows into L1
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            if (ncell[c] < 0) continue;
            const T *S = P.S + (size_t)ncell[c] * 3 * NP;
            prefetch_l1(S);
            prefetch_l1(S + 3 * NP - 1);
            if constexpr (3 * NP * sizeof(T) > 128) prefetch_l1(S + 128 / sizeof(T));
            cell[c] = ncell[c];
        }
        beg = nbeg;
        end = nend;
    }
    if (sing) atomicAdd(P.singular, sing);
}

template <typename T, int DEG, bool PRECOMP, int CPT, int TPG, int GMAX, bool CH>
__global__ void __launch_bounds__(GMAX * TPG) sweep_ring_kernel(SweepParams<T> P, RingParams Q) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ring_body<T, DEG, PRECOMP, CPT, TPG, GMAX, CH>(P, Q, (int)blockIdx.x, smem_raw);
}

// Many cases of one degree in one launch: the blocks of case k are
// block0[k] .. block0[k] + nblocks[k] - 1 (cases ordered by block0); each
// block copies its case's parameters into shared memory and sweeps one of
// its velocities.  The launch's shared memory is the largest ring of the
// cases; each case's far slots start after its own ring.
struct RingCase {
    SweepParams<float> P;
    RingParams Q;
    int block0, nblocks;
};

template <int DEG, int CPT, int TPG, int GMAX>
__global__ void __launch_bounds__(GMAX * TPG) sweep_ring_batch_kernel(const RingCase *cases, int ncases) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ RingCase sc;
    if (threadIdx.x == 0) {
        int lo = 0, hi = ncases - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (cases[mid].block0 <= (int)blockIdx.x) lo = mid;
            else hi = mid - 1;
        }
        sc = cases[lo];
    }
    __syncthreads();
    ring_body<float, DEG, false, CPT, TPG, GMAX, true>(sc.P, sc.Q, (int)blockIdx.x - sc.block0, smem_raw);
}

template <typename T, int DEG, bool PRE, int TPG, int GMAX>
static int ring_launch_cpt(pbte_ctx *c, const SweepParams<T> &P, const RingParams &Q, int cpt, size_t shm,
                           cudaStream_t s) {
    const int threads = Q.groups * TPG;
    const bool chunked = c->ring_W > cpt * TPG;
    auto go = [&](auto kern) {
        if (shm > 48 * 1024 &&
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm) != cudaSuccess)
            return PBTE_ERR_CUDA;
        kern<<<Q.unfold ? c->ndir : c->n_udir, threads, shm, s>>>(P, Q);
        return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
    };
    switch (cpt) {
        case 1:
            if (chunked) return go(sweep_ring_kernel<T, DEG, PRE, 1, TPG, GMAX, true>);
            return go(sweep_ring_kernel<T, DEG, PRE, 1, TPG, GMAX, false>);
        case 2:
            if constexpr (DEG <= 2 && TPG == 64) {
                if (chunked) return go(sweep_ring_kernel<T, DEG, PRE, 2, TPG, GMAX, true>);
                return go(sweep_ring_kernel<T, DEG, PRE, 2, TPG, GMAX, false>);
            }
            return PBTE_ERR_UNSUPPORTED;
        case 4:
            // four elements per thread cover levels up to 256 wide: never chunked
            if constexpr (sizeof(T) == 4 && DEG <= 2 && TPG == 64 && GMAX <= 4)
                if (!chunked) return go(sweep_ring_kernel<T, DEG, PRE, 4, TPG, GMAX, false>);
            return PBTE_ERR_UNSUPPORTED;
        default: return PBTE_ERR_UNSUPPORTED;
    }
}

// Returns PBTE_ERR_UNSUPPORTED when the ring form does not fit (the caller
// then uses the level-serial kernel): degree above 3, or a ring that does not
// fit in shared memory.  Block shapes compiled: groups of 64 with up to four
// groups (1, 2 or 4 elements per thread in registers); for DEG <= 2 also up
// to eight groups of 64 (1 or 2 elements per thread) and up to four groups of
// 128 (1 element per thread), the 512-thread shapes whose operators fit the
// 128 registers such a block allows.  A level wider than a group's elements
// in registers runs in chunks (sweep_ring_kernel), so any level width is
// served.  A requested shape that is not compiled for the mesh falls back to
// four groups of 64.
template <typename T, bool PRE>
int launch_ring(pbte_ctx *c, const SweepParams<T> &P, cudaStream_t s) {
    if (c->deg > 3 || c->ring_W <= 0) return PBTE_ERR_UNSUPPORTED;
    auto cpt_for = [&](int width) {
        const int k = (c->ring_W + width - 1) / width;
        return k == 3 ? 4 : k;
    };
    int width = c->ring_width == 128 ? 128 : 64;
    int groups = c->ring_groups > 0 ? std::min(c->ring_groups, kMaxGroups) : 4;
    if (c->ring_groups == 0 && c->ring_width == 0 && c->deg <= 2) {
        // measured defaults (square cavities, P1/P2, 256-512 ordinates):
        // levels up to 64 wide take eight groups of 64 in FP32 (four in FP64,
        // whose operators need twice the registers), levels up to 128 wide
        // four groups of 128, wider levels two groups of 128 in chunks (two
        // 256-thread blocks fit an SM, so all the 256 velocities of a
        // 512-ordinate case run at once: 3.3 ms against 4.9 with four groups
        // on the 256 x 256 square)
        if (c->ring_W <= 64) groups = sizeof(T) == 4 ? 8 : 4;
        else if (c->ring_W <= 128) width = 128;
        else { width = 128; groups = 2; }
    }
    if (width == 128 && (c->deg > 2 || groups > 4)) width = 64;
    if (groups > 4 && c->deg > 2) groups = 4;
    // elements per thread held in registers: what the level needs, up to what
    // the shape is compiled for (chunks cover the rest)
    int cpt = cpt_for(width);
    int cpt_max = 1;
    if (width == 64 && c->deg <= 2) cpt_max = (sizeof(T) == 4 && groups <= 4 && cpt == 4) ? 4 : 2;
    cpt = std::min(cpt, cpt_max);
    const size_t ring_vals = (size_t)c->ring_R * c->ring_W * c->nd;
    const size_t shm = sizeof(T) * ((size_t)6 * c->nd * c->nd + ring_vals + (size_t)c->far_max * c->nd);
    if (shm > 200 * 1024) return PBTE_ERR_UNSUPPORTED;
    const void *rf = sizeof(T) == 4 ? (const void *)c->d_rf32 : (const void *)c->d_rf64;
    RingParams Q{rf, c->d_ri, (int64_t)c->nclass * c->n_tris, c->d_class_W, c->d_class_R,
                 c->d_udir_rep, c->d_udir_twin, groups, (int)ring_vals, c->has_periodic ? 1 : 0};
    if (Q.unfold && P.by_udir) return PBTE_ERR_UNSUPPORTED;
    if (width == 128) {
        switch (c->deg) {
            case 1: return ring_launch_cpt<T, 1, PRE, 128, 4>(c, P, Q, cpt, shm, s);
            case 2: return ring_launch_cpt<T, 2, PRE, 128, 4>(c, P, Q, cpt, shm, s);
            default: return PBTE_ERR_UNSUPPORTED;
        }
    }
    if (groups > 4) {
        switch (c->deg) {
            case 1: return ring_launch_cpt<T, 1, PRE, 64, 8>(c, P, Q, cpt, shm, s);
            case 2: return ring_launch_cpt<T, 2, PRE, 64, 8>(c, P, Q, cpt, shm, s);
            default: return PBTE_ERR_UNSUPPORTED;
        }
    }
    switch (c->deg) {
        case 1: return ring_launch_cpt<T, 1, PRE, 64, 4>(c, P, Q, cpt, shm, s);
        case 2: return ring_launch_cpt<T, 2, PRE, 64, 4>(c, P, Q, cpt, shm, s);
        case 3: return ring_launch_cpt<T, 3, PRE, 64, 4>(c, P, Q, cpt, shm, s);
        default: return PBTE_ERR_UNSUPPORTED;
    }
}

template int launch_ring<double, false>(pbte_ctx *, const SweepParams<double> &, cudaStream_t);
template int launch_ring<double, true>(pbte_ctx *, const SweepParams<double> &, cudaStream_t);
template int launch_ring<float, false>(pbte_ctx *, const SweepParams<float> &, cudaStream_t);
template int launch_ring<float, true>(pbte_ctx *, const SweepParams<float> &, cudaStream_t);

// FP32 factors for the ring sweep, one thread per (distinct in-plane
// velocity u, sweep position p): the FP32 records and the same arithmetic
// as the sweep's in-register factorisation (assemble<float>, no
// interchanges, __frcp_rn of the pivot), so a sweep with stored factors gives
// the bits of one without.
template <int DEG>
__global__ void factorise32_kernel(SweepParams<float> P, const float *__restrict__ rf, int64_t M,
                                   const int32_t *__restrict__ udir_rep, int n_udir, float *__restrict__ lu_out) {
    constexpr int NP = Shape<DEG>::NP;
    __shared__ float sref[6 * NP * NP];
    for (int k = threadIdx.x; k < 6 * NP * NP; k += blockDim.x) sref[k] = P.ref[k];
    __syncthreads();
    const size_t total = (size_t)n_udir * P.nt;
    int sing = 0;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int u = (int)(t / P.nt), p = (int)(t % P.nt);
        const int d = udir_rep[u];
        const int64_t k = (int64_t)P.dir_class[d] * P.nt + p;
        const float cx = (float)P.cx[d], cy = (float)P.cy[d];
        Geo<float> r;
        float s[3];
#pragma unroll
        for (int il = 0; il < 3; ++il) {
            r.es[il] = rf[(kREs + il) * M + k];
            s[il] = cx * rf[(kRNx + il) * M + k] + cy * rf[(kRNy + il) * M + k];
        }
        r.area2 = rf[kRA2 * M + k];
        r.gxa = rf[kRGxa * M + k];
        r.gxb = rf[kRGxb * M + k];
        r.gya = rf[kRGya * M + k];
        r.gyb = rf[kRGyb * M + k];
        float A[NP][NP];
        assemble<float, DEG>(sref, r, cx, cy, P.inv_tau_c, s, A);
#pragma unroll
        for (int kk = 0; kk < NP; ++kk) {
            sing += (A[kk][kk] == 0.0f);
            const float rr = __frcp_rn(A[kk][kk]);
#pragma unroll
            for (int ii = kk + 1; ii < NP; ++ii) {
                A[ii][kk] *= rr;
#pragma unroll
                for (int j = kk + 1; j < NP; ++j) A[ii][j] -= A[ii][kk] * A[kk][j];
            }
            A[kk][kk] = rr;
        }
        float *o = lu_out + factor_base(u, p, P.nt, NP * NP);
#pragma unroll
        for (int m = 0; m < NP; ++m)
#pragma unroll
            for (int l = 0; l < NP; ++l) o[32 * (m * NP + l)] = A[m][l];
    }
    if (sing) atomicAdd(P.singular, sing);
}

int launch_factorise32(pbte_ctx *c, cudaStream_t s) {
    if (c->deg > 3 || !c->d_lu32) return PBTE_ERR_UNSUPPORTED;
    SweepParams<float> P{};
    P.ref = c->d_ref32;
    P.cx = c->d_cx;
    P.cy = c->d_cy;
    P.dir_class = c->d_dir_class;
    P.nt = c->n_tris;
    P.inv_tau_c = (float)(1.0 / c->tau_c);
    P.singular = c->d_singular;
    const int th = 128;
    const size_t total = (size_t)c->n_udir * c->n_tris;
    const int bl = (int)std::min<size_t>((total + th - 1) / th, 152 * 16);
    const int64_t M = (int64_t)c->nclass * c->n_tris;
    switch (c->deg) {
        case 1: factorise32_kernel<1><<<bl, th, 0, s>>>(P, c->d_rf32, M, c->d_udir_rep, c->n_udir, c->d_lu32); break;
        case 2: factorise32_kernel<2><<<bl, th, 0, s>>>(P, c->d_rf32, M, c->d_udir_rep, c->n_udir, c->d_lu32); break;
        case 3: factorise32_kernel<3><<<bl, th, 0, s>>>(P, c->d_rf32, M, c->d_udir_rep, c->n_udir, c->d_lu32); break;
        default: return PBTE_ERR_UNSUPPORTED;
    }
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

}  // namespace pbte

// ---------------------------------------------------------------------------
// Many cases' folded FP32 sweeps in one launch per degree (pbte_sweep_batch_*)
struct pbte_sweep_batch {
    struct Group {
        int deg = 0, tpg = 64, groups = 4, nblocks = 0;
        size_t shm = 0;
        pbte::RingCase *d_cases = nullptr;
        int ncases = 0;
    };
    std::vector<Group> groups;
    std::vector<pbte_batch_item> items;
};

namespace pbte {
namespace {

template <int DEG, int CPT, int TPG, int GMAX>
int batch_go(const pbte_sweep_batch::Group &g, cudaStream_t s) {
    auto kern = sweep_ring_batch_kernel<DEG, CPT, TPG, GMAX>;
    if (g.shm > 48 * 1024 &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.shm) != cudaSuccess)
        return PBTE_ERR_CUDA;
    kern<<<g.nblocks, g.groups * TPG, g.shm, s>>>(g.d_cases, g.ncases);
    return cudaGetLastError() == cudaSuccess ? PBTE_OK : PBTE_ERR_CUDA;
}

int batch_launch(const pbte_sweep_batch::Group &g, cudaStream_t s) {
    if (g.tpg == 128) {
        if (g.deg == 1) return batch_go<1, 1, 128, 4>(g, s);
        if (g.deg == 2) return batch_go<2, 1, 128, 4>(g, s);
    } else if (g.groups > 4) {
        if (g.deg == 1) return batch_go<1, 1, 64, 8>(g, s);
        if (g.deg == 2) return batch_go<2, 1, 64, 8>(g, s);
    } else {
        if (g.deg == 1) return batch_go<1, 1, 64, 4>(g, s);
        if (g.deg == 2) return batch_go<2, 1, 64, 4>(g, s);
        if (g.deg == 3) return batch_go<3, 1, 64, 4>(g, s);
    }
    return PBTE_ERR_UNSUPPORTED;
}

}  // namespace
}  // namespace pbte

extern "C" int pbte_sweep_batch_destroy(pbte_sweep_batch *b) {
    if (!b) return PBTE_OK;
    for (auto &g : b->groups)
        if (g.d_cases) cudaFree(g.d_cases);
    delete b;
    return PBTE_OK;
}

static int batch_create_impl(int32_t n, const pbte_batch_item *items, int32_t groups, int32_t width,
                             pbte_sweep_batch **out) {
    if (!out || n <= 0 || !items || groups < 1 || groups > pbte::kMaxGroups || (width != 64 && width != 128))
        return PBTE_ERR_ARG;
    *out = nullptr;
    const int dev = items[0].ctx ? items[0].ctx->device : -1;
    for (int i = 0; i < n; ++i) {
        const pbte_batch_item &it = items[i];
        if (!it.ctx || !it.ts || !it.qxs || !it.qys || !it.vdf32 || (it.ctx->n_wall_ad && !it.flux_wall))
            return PBTE_ERR_ARG;
        if (it.ctx->device != dev) return PBTE_ERR_ARG;
        if (it.ctx->has_periodic || it.ctx->deg > 3 || it.ctx->ring_W <= 0) return PBTE_ERR_UNSUPPORTED;
    }
    auto *b = new pbte_sweep_batch();
    b->items.assign(items, items + n);
    for (int deg = 1; deg <= 3; ++deg) {
        pbte_sweep_batch::Group g;
        g.deg = deg;
        g.tpg = (deg <= 2 && width == 128) ? 128 : 64;
        g.groups = (deg == 3 || g.tpg == 128) ? std::min(groups, 4) : groups;
        std::vector<pbte::RingCase> cases;
        for (int i = 0; i < n; ++i) {
            pbte_ctx *c = items[i].ctx;
            if (c->deg != deg) continue;
            pbte::RingCase rc{};
            rc.P = pbte::fold_params32(c, items[i].vdf32, items[i].flux_wall, items[i].wall_scale, items[i].done);
            const size_t ring_vals = (size_t)c->ring_R * c->ring_W * c->nd;
            rc.Q = pbte::RingParams{c->d_rf32, c->d_ri, (int64_t)c->nclass * c->n_tris, c->d_class_W, c->d_class_R,
                                    c->d_udir_rep, c->d_udir_twin, g.groups, (int)ring_vals, 0};
            rc.block0 = g.nblocks;
            rc.nblocks = c->n_udir;
            g.nblocks += c->n_udir;
            g.shm = std::max(g.shm, sizeof(float) * ((size_t)6 * c->nd * c->nd + ring_vals + (size_t)c->far_max * c->nd));
            cases.push_back(rc);
        }
        if (cases.empty()) continue;
        if (g.shm > 200 * 1024) {
            pbte_sweep_batch_destroy(b);
            return PBTE_ERR_UNSUPPORTED;
        }
        g.ncases = (int)cases.size();
        if (cudaMalloc((void **)&g.d_cases, cases.size() * sizeof(pbte::RingCase)) != cudaSuccess) {
            pbte_sweep_batch_destroy(b);
            return PBTE_ERR_NOMEM;
        }
        b->groups.push_back(g);
        if (cudaMemcpy(g.d_cases, cases.data(), cases.size() * sizeof(pbte::RingCase), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
            pbte_sweep_batch_destroy(b);
            return PBTE_ERR_CUDA;
        }
    }
    *out = b;
    return PBTE_OK;
}

extern "C" int pbte_sweep_batch_create(int32_t n, const pbte_batch_item *items, int32_t groups, int32_t width,
                                       pbte_sweep_batch **out) {
    try {
        return batch_create_impl(n, items, groups, width, out);
    } catch (...) {
        if (out) *out = nullptr;
        return PBTE_ERR_NOMEM;
    }
}

extern "C" int pbte_sweep_batch_run(pbte_sweep_batch *b, int with_sources, void *stream) {
    if (!b) return PBTE_ERR_ARG;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (with_sources)
        for (const auto &it : b->items) {
            const int rc = pbte::launch_sources(it.ctx, it.ts, it.qxs, it.qys, true, s);
            if (rc) return rc;
        }
    for (const auto &g : b->groups) {
        const int rc = pbte::batch_launch(g, s);
        if (rc) return rc;
    }
    return PBTE_OK;
}
