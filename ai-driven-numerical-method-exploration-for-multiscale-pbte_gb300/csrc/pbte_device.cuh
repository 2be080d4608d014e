// Device helpers shared by the sweep kernels: element shape tables, kernel
// parameters, operator assembly, right-hand side, in-register LU.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "pbte_internal.cuh"

namespace pbte {

constexpr int kSweepThreads = 128;

template <int DEG>
struct Shape {
    static constexpr int NP = (DEG + 1) * (DEG + 2) / 2;
    static constexpr int NF = DEG + 1;
    __host__ __device__ static constexpr int idx(int i, int j) { return j * (DEG + 1) - j * (j - 1) / 2 + i; }
    // element DOF of the b-th node along local edge il (edges walk node1->2, 2->3, 3->1)
    __host__ __device__ static constexpr int edof(int il, int b) {
        return il == 0 ? idx(b, 0) : (il == 1 ? idx(DEG - b, b) : idx(0, DEG - b));
    }
};

__device__ __forceinline__ bool stopped(const int32_t *done) { return done != nullptr && *(volatile const int32_t *)done != 0; }

template <typename T>
struct SweepParams {
    const CellRec<T> *cells;
    const T *ref;  // [6][NP*NP]
    const T *S;    // [n_tris][3][NP]
    T *vdf;        // [ndir][n_tris][NP]
    const double *flux_wall;
    // periodic inflow not read from vdf: row pslot[face] (or face, when pslot
    // is null) of pbuf, which has pb_rows rows of NP values per ordinate
    const double *pbuf;
    const int32_t *pslot;
    int pb_rows;
    int use_pbuf;             // 1: every periodic face reads pbuf (explicit state)
    const uint8_t *fresh;     // [nclass][nt] periodic faces read from vdf when use_pbuf == 0
    const double *cx, *cy;
    const int32_t *dir_class, *class_off, *class_nlev, *lvl_ptr, *lvl_cells;
    const double *lu;       // stored factors, factor_base() layout
    const int8_t *piv;
    const float *lu32;      // stored FP32 factors (no interchanges), factor_base() layout
    const int32_t *udir_of; // ordinate -> distinct in-plane velocity (factor owner)
    int store_twin;         // ring sweep: also store the z-mirror twin's copy (0: folded consumers)
    int by_udir;            // ring sweep: row of the distinct velocity u instead of the ordinate d
    int32_t *singular;
    const int32_t *done;
    int nt, n_faces;
    T inv_tau_c, ca, cb, wall_scale;
};

// Assemble the element operator.  Rec: anything with the geometry members
// of CellRec (area2, gxa, gxb, gya, gyb, es[3]).
template <typename T, int DEG, typename Rec>
__device__ __forceinline__ void assemble(const T *sref, const Rec &r, T cx, T cy, T inv_tau_c,
                                         const T (&s)[3], T (&A)[Shape<DEG>::NP][Shape<DEG>::NP]) {
    constexpr int NP = Shape<DEG>::NP, NF = Shape<DEG>::NF;
    const T p = r.area2 * inv_tau_c;
    const T q = -r.area2 * (cx * r.gxa + cy * r.gya);
    const T w = -r.area2 * (cx * r.gxb + cy * r.gyb);
#pragma unroll
    for (int m = 0; m < NP; ++m)
#pragma unroll
        for (int l = 0; l < NP; ++l)
            A[m][l] = p * sref[m * NP + l] + q * sref[NP * NP + m * NP + l] + w * sref[2 * NP * NP + m * NP + l];
#pragma unroll
    for (int il = 0; il < 3; ++il) {
        const T sc = s[il] > T(0) ? s[il] * r.es[il] : T(0);
        const T *R = sref + (3 + il) * NP * NP;
#pragma unroll
        for (int a = 0; a < NF; ++a)
#pragma unroll
            for (int b = 0; b < NF; ++b) {
                const int ma = Shape<DEG>::edof(il, a), lb = Shape<DEG>::edof(il, b);
                A[ma][lb] += sc * R[ma * NP + lb];
            }
    }
}

// Right-hand side: Callaway source from the moment sources plus the upwind
// inflow.  fresh: bit il set when a periodic face il reads the partner's row
// of f (unless P.use_pbuf), else it reads pbuf.
template <typename T, int DEG>
__device__ __forceinline__ void rhs(const SweepParams<T> &P, const T *sref, const CellRec<T> &r, int i,
                                    int d, T cx, T cy, const T (&s)[3], const T *f,
                                    T (&b)[Shape<DEG>::NP], unsigned fresh) {
    constexpr int NP = Shape<DEG>::NP, NF = Shape<DEG>::NF;
    const T *S = P.S + (size_t)i * 3 * NP;
#pragma unroll
    for (int m = 0; m < NP; ++m) b[m] = P.ca * S[m] + P.cb * (cx * S[NP + m] + cy * S[2 * NP + m]);
#pragma unroll
    for (int il = 0; il < 3; ++il) {
        if (!(s[il] < T(0))) continue;
        const T w = s[il];
        const T *R = sref + (3 + il) * NP * NP;
        const int kind = r.kind[il];
        if (kind == 0 || kind == 3) {
            T g[NF];
            if (kind == 3 && (P.use_pbuf || !((fresh >> il) & 1u))) {
                const int row = P.pslot ? P.pslot[r.face[il]] : r.face[il];
                const double *pb = P.pbuf + ((size_t)d * P.pb_rows + row) * NP;
#pragma unroll
                for (int bb = 0; bb < NF; ++bb) g[bb] = (T)pb[r.emap[il][bb]];
            } else {
                const T *fn = f + (size_t)r.upw[il] * NP;
#pragma unroll
                for (int bb = 0; bb < NF; ++bb) g[bb] = fn[r.emap[il][bb]];
            }
            const T sc = w * r.es[il];
#pragma unroll
            for (int a = 0; a < NF; ++a) {
                const int ma = Shape<DEG>::edof(il, a);
                T acc = T(0);
#pragma unroll
                for (int bb = 0; bb < NF; ++bb) acc += R[ma * NP + Shape<DEG>::edof(il, bb)] * g[bb];
                b[ma] -= sc * acc;
            }
        } else if (kind == 1) {
            const T sc = w * r.bval[il] * P.wall_scale * r.es[il];
#pragma unroll
            for (int a = 0; a < NF; ++a) {
                const int ma = Shape<DEG>::edof(il, a);
                T rs = T(0);
#pragma unroll
                for (int bb = 0; bb < NF; ++bb) rs += R[ma * NP + Shape<DEG>::edof(il, bb)];
                b[ma] -= sc * rs;
            }
        } else {
            const double *fw = P.flux_wall + (size_t)r.face[il] * NP;
#pragma unroll
            for (int m = 0; m < NP; ++m) b[m] -= w * (-(T)fw[m]);
        }
    }
}

// LU with partial pivoting (first maximum, as DGETF2) applied to b on the fly,
// then back substitution; returns the number of zero pivots.
template <typename T, int N>
__device__ __forceinline__ int lu_solve(T (&A)[N][N], T (&b)[N]) {
    int sing = 0;
    T rinv[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        T big = fabs(A[k][k]);
        int p = k;
#pragma unroll
        for (int i = k + 1; i < N; ++i) {
            const T v = fabs(A[i][k]);
            if (v > big) { big = v; p = i; }
        }
#pragma unroll
        for (int i = k + 1; i < N; ++i) {
            if (p == i) {
#pragma unroll
                for (int j = 0; j < N; ++j) { const T t = A[k][j]; A[k][j] = A[i][j]; A[i][j] = t; }
                const T t = b[k]; b[k] = b[i]; b[i] = t;
            }
        }
        sing += (A[k][k] == T(0));
        rinv[k] = T(1) / A[k][k];
#pragma unroll
        for (int i = k + 1; i < N; ++i) {
            const T l = A[i][k] * rinv[k];
#pragma unroll
            for (int j = k + 1; j < N; ++j) A[i][j] -= l * A[k][j];
            b[i] -= l * b[k];
        }
    }
#pragma unroll
    for (int k = N - 1; k >= 0; --k) {
        b[k] *= rinv[k];
#pragma unroll
        for (int i = 0; i < k; ++i) b[i] -= b[k] * A[i][k];
    }
    return sing;
}

// ring-pipelined sweep (pbte_sweep.cu); PBTE_ERR_UNSUPPORTED when it does not fit
template <typename T, bool PRE>
int launch_ring(pbte_ctx *c, const SweepParams<T> &P, cudaStream_t s);
// the parameters of a folded FP32 sweep (rows by distinct velocity, factored
// in registers) of context c, with `done` as its stop flag
SweepParams<float> fold_params32(pbte_ctx *c, float *vdf32, const double *fw, double wall_scale,
                                 const int32_t *done);

}  // namespace pbte
