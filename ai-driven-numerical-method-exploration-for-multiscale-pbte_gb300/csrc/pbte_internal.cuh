// Internal definitions shared by the translation units of libpbte_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <vector>

#include "pbte_gb300.h"

namespace pbte {

// device bytes held by all live contexts (pbte_device_bytes_live)
extern std::atomic<long long> g_live_bytes;

constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr int kMaxNf = 5;   // deg <= 4

// Per-element record read by the sweep: the compact operator description of
// one triangle plus its three faces.  One 16-byte-aligned struct per element
// so a thread fetches it in a few wide loads.
template <typename T>
struct alignas(16) CellRec {
    T area2;        // 2 * area
    T gxa, gxb;     // d(xi)/dx, d(eta)/dx  (gx = area2 (gxa ref_dx + gxb ref_dy))
    T gya, gyb;     // d(xi)/dy, d(eta)/dy
    T es[3];        // edge scale: len12, len23/sqrt2, len31
    T nx[3], ny[3]; // outward unit normals
    T bval[3];      // cv/(4 pi) T_wall on thermalising edges, else 0
    int32_t face[3];
    int32_t upw[3];         // upwind element across the edge (neighbour or periodic partner), -1 on walls
    int8_t kind[3];         // 0 interior, 1 thermalising, 2 adiabatic, 3 periodic
    int8_t emap[3][kMaxNf]; // neighbour DOF facing each of this element's edge DOFs
};

// Element records of the ring sweep, field-major: field f of the element at
// position k of a direction class's sweep order (k in [cls * n_tris,
// (cls + 1) * n_tris)) is at f * stride + k, so a warp reading one field of
// consecutive positions makes one coalesced access.
//   real fields (T):  area2, gxa, gxb, gya, gyb, es[3], nx[3], ny[3], bval[3]
//   int fields:       cell, far_out, up[3], emp[3], face[3], kind (3 bytes)
// up[il]: -1 no in-sweep inflow; >= 0 slot of the near ring
// ((level % R) * W + position); <= -2 far slot -(up + 2).
// far_out: far slot this element's values must also be kept in, or -1.
// emp[il]: emap[il][0..nf-1] packed four bits each (nd <= 15).
// kind: kind[il] in byte il; the records add kind 4, a periodic face whose
// partner precedes the element in the reference's sweep order (its inflow is
// this sweep's value, read like an interior neighbour's), while kind 3 there
// is a periodic face read from the previous sweep's values.
enum RecReal { kRA2 = 0, kRGxa, kRGxb, kRGya, kRGyb, kREs, kRNx = kREs + 3, kRNy = kRNx + 3,
               kRBval = kRNy + 3, kNumRecReal = kRBval + 3 };
enum RecInt { kICell = 0, kIFarOut, kIUp, kIEmp = kIUp + 3, kIFace = kIEmp + 3, kIKind = kIFace + 3,
              kNumRecInt };

// Stored FP64 factors are kept once per distinct in-plane velocity u (z-mirror
// twins share them), in the direction class's sweep order and interleaved by
// 32 positions: entry e (of NP*NP, or of NP pivots) of the element at sweep
// position p (0 <= p < nt) is at factor_base(u, p, nt, n) + 32 * e, n = NP*NP
// or NP.  A warp reading one entry of consecutive positions makes one
// coalesced access.
__host__ __device__ __forceinline__ size_t factor_base(int u, int p, int nt, int n) {
    const int nblk = (nt + 31) >> 5;
    return ((size_t)u * nblk + (size_t)(p >> 5)) * (size_t)n * 32 + (size_t)(p & 31);
}
__host__ __device__ __forceinline__ size_t factor_count(int n_udir, int nt, int n) {
    return (size_t)n_udir * (size_t)((nt + 31) >> 5) * (size_t)n * 32;
}

struct WallFace {
    int32_t face, tri, lfc, pad;
    double nx, ny;  // inward normal (-n_out of the adjacent element)
};

}  // namespace pbte

struct pbte_ctx {
    int n_tris = 0, n_faces = 0, nd = 0, nf = 0, ndir = 0, nbc = 0, deg = 0;
    int device = -1;   // the CUDA device current when the context was created
    double cv = 1, vg = 1, tau_r = 1, tau_n = 1, tau_c = 1;
    std::vector<double> h_cx, h_cy, h_w;
    bool has_periodic = false;

    // device data
    double *d_cx = nullptr, *d_cy = nullptr, *d_w = nullptr;
    pbte::CellRec<double> *d_cells64 = nullptr;
    pbte::CellRec<float> *d_cells32 = nullptr;
    double *d_ref64 = nullptr;   // [6][nd*nd]: mass, dx, dy, edge0, edge1, edge2
    float *d_ref32 = nullptr;
    int32_t *d_edofs = nullptr;  // [3][nf]
    int32_t *d_dir_class = nullptr;
    int32_t *d_class_lvl_off = nullptr;  // [nclass]: offset of the class's level pointer block
    int32_t *d_class_nlev = nullptr;     // [nclass]
    int32_t *d_lvl_ptr = nullptr;        // concatenated level pointers (into d_lvl_cells)
    int32_t *d_lvl_cells = nullptr;      // [nclass][n_tris]
    int nclass = 0, nlev_max = 0;
    double *d_int_tri = nullptr;
    int n_wall_ad = 0;
    pbte::WallFace *d_wall_ad = nullptr;
    double *d_S64 = nullptr;  // [3][nd][n_tris] moment sources of the current sweep
    float *d_S32 = nullptr;
    double *d_lu = nullptr;   // precomputed factors (optional), factor_base() layout
    int8_t *d_piv = nullptr;
    // FP32 factors for the FP32 sweeps (optional; no row interchanges, 1/U_kk
    // on the diagonal), factor_base() layout, made by pbte_factorise_f32 with
    // the FP32 sweep's own in-register arithmetic
    float *d_lu32 = nullptr;
    double *d_red = nullptr;  // reduction scratch
    int32_t *d_singular = nullptr;
    const int32_t *done = nullptr;  // optional device stop flag
    size_t device_bytes = 0;
    // ring-buffered sweep: per-class upwind ring slots, widest level, deepest gap
    int32_t *d_up_slot = nullptr;   // [nclass][n_tris in level order][3], -1: no in-sweep inflow
    int32_t *d_class_W = nullptr, *d_class_R = nullptr;
    int ring_W = 0, ring_R = 0;
    // one sweep per distinct in-plane velocity: representative ordinate and its z-twin (-1 if none)
    int32_t *d_udir_rep = nullptr, *d_udir_twin = nullptr;
    int32_t *d_udir_of = nullptr;   // [ndir]: the distinct velocity an ordinate belongs to
    int n_udir = 0;
    // per distinct velocity, FP32: summed weight of the ordinate and its twin, cx, cy
    float *d_uw32 = nullptr, *d_ucx32 = nullptr, *d_ucy32 = nullptr;
    double *d_uw64 = nullptr, *d_ucx64 = nullptr, *d_ucy64 = nullptr;
    int sweep_variant = 0;          // 0 automatic, 1 level-serial, 2 ring pipeline
    int ring_groups = 0;            // thread groups of the ring pipeline (0: default)
    int ring_width = 0;             // threads per group of the ring pipeline (0: 64)
    // per-class records in sweep order, field-major with stride nclass * n_tris
    // (RecReal / RecInt), and the far-slot count
    double *d_rf64 = nullptr;
    float *d_rf32 = nullptr;
    int32_t *d_ri = nullptr;
    int far_max = 0;
    double *d_mom_part = nullptr;   // [ceil(ndir/32)][3][n_tris*ndof] moment partial sums
    float *d_cx32 = nullptr, *d_cy32 = nullptr, *d_w32 = nullptr;   // ordinates in FP32
    // Periodic faces.  pybte's source-iteration sweep reads the partner's
    // current values, i.e. this sweep's when the partner comes earlier in the
    // direction's TRI_ORDER ("fresh": a dependency of the schedule) and the
    // previous sweep's otherwise ("lagged": read from a snapshot taken before
    // the sweep).  Sweeps over periodic faces are not z-twin folded: twins
    // may see different partner values.
    uint8_t *d_fresh = nullptr;     // [nclass][n_tris]: bit il set when face il reads a fresh partner
    int n_pfaces = 0;               // periodic faces, in increasing face index
    int32_t *d_pface = nullptr, *d_ptri = nullptr;  // [n_pfaces]: face, partner element behind it
    int32_t *d_pslot = nullptr;     // [n_faces]: row of a periodic face in the compact buffers, else -1
    double *d_psnap = nullptr;      // [ndir][n_pfaces][nd]: partner values before a source-iteration sweep
    double *d_gsis = nullptr;       // [4][n_tris * nd]: GSIS moment rows / correction coefficients
    uint32_t *d_tickets = nullptr;  // [ceil(n_tris / 32)]: last-block tickets of the folded epilogue (kept 0)
};

// launchers (pbte_kernels.cu)
namespace pbte {
int launch_sources(pbte_ctx *c, const double *ts, const double *qxs, const double *qys, bool f32,
                   cudaStream_t s);
int launch_sweep64(pbte_ctx *c, double *vdf, const double *flux_wall, const double *pbuf,
                   int use_pbuf, cudaStream_t s);
int launch_sweep32(pbte_ctx *c, float *vdf32, const double *flux_wall, double wall_scale,
                   cudaStream_t s, bool store_twin = true, bool by_udir = false);
// the FP32 fixed-point product with z-mirror twins folded (one copy per
// in-plane velocity written and read): sources, sweep, moments, emission
// with_sources = false: the moment sources of the inputs are already in
// d_S32 (left by launch_next_basis_sources)
int launch_fixed_point32(pbte_ctx *c, const double *ts, const double *qxs, const double *qys,
                         const double *fw_in, double wall_scale, float *vdf32, double *ts_out,
                         double *qxs_out, double *qys_out, double *fw_out, double *temp, double *qx,
                         double *qy, cudaStream_t s, bool with_sources = true);
// moments, element integrals and wall emission of a folded FP32 distribution
int launch_fold_epilogue32(pbte_ctx *c, const float *vdf32, double *ts_out, double *qxs_out, double *qys_out,
                           double *fw_out, double *temp, double *qx, double *qy, cudaStream_t s);
// pbte_arnoldi_column_f32 + pbte_gmres_givens for column rows - 1, the
// rotation run by the last block of the CGS2 norm pass (pbte_krylov.cu)
int arnoldi_column_givens_f32(const float *Q, int64_t ldq, int32_t rows, const double *uout, const double *g,
                              float *w, int64_t n, double *h, double *scratch, int64_t scratch_len, double *R,
                              int32_t ldr, double *cs, double *sn, double *gam, const double *tol_abs,
                              int32_t *state, double *hist, cudaStream_t s);
// GMRES next basis vector (FP32 basis) plus the moment sources of the next
// FP32 product into d_S32; PBTE_ERR_UNSUPPORTED for N_p other than 3, 6, 10
int launch_next_basis_sources(pbte_ctx *c, int j, const float *w, const double *h, float *Q, int64_t ldq,
                              double *uin, int64_t n, const int32_t *state, cudaStream_t s);
int launch_factorise(pbte_ctx *c, cudaStream_t s);
int launch_factorise32(pbte_ctx *c, cudaStream_t s);
int launch_moments64(pbte_ctx *c, const double *vdf, double *ts, double *qxs, double *qys,
                     double *temp, double *qx, double *qy, cudaStream_t s);
int launch_moments32(pbte_ctx *c, const float *vdf, double *ts, double *qxs, double *qys,
                     double *temp, double *qx, double *qy, cudaStream_t s);
int launch_wall_flux64(pbte_ctx *c, const double *vdf, double *fw, cudaStream_t s);
int launch_wall_flux32(pbte_ctx *c, const float *vdf, double *fw, cudaStream_t s);
int launch_residual(pbte_ctx *c, const double *temp, double *t_old, double *out, cudaStream_t s);
int launch_residual_check(pbte_ctx *c, const double *res, double tol, int64_t tmax, int32_t *done,
                          int64_t *count, double *hist, int64_t hist_cap, cudaStream_t s);
int launch_transport_residual(pbte_ctx *c, const double *ts, const double *qxs, const double *qys,
                              const double *vdf, const double *fw, const double *pbuf,
                              double *num, double *den, cudaStream_t s);
int launch_transport_residual_scratch(pbte_ctx *c, const double *ts, const double *qxs, const double *qys,
                                      const double *vdf, const double *fw, double *num, double *den,
                                      double *S, cudaStream_t s);
int launch_hot_source(pbte_ctx *c, const double *vdf, double tc5, double *work, cudaStream_t s);
int launch_gsis_hot_apply(pbte_ctx *c, const pbte_gsis_ops *o, const double *vdf, double tc5, double *aa_src,
                          cudaStream_t s);
// one step of the FP32 GSIS product on the folded FP32 distribution: 0 hot
// source with the inverses, 1 kinetic wall traces, 2 damped correction
int launch_gsis_product32(pbte_ctx *c, const pbte_gsis_ops *o, int step, float *vdf32, double tc5,
                          const double *tri_fc_fc, int nk, const int32_t *tri_list, const int32_t *lfc_list,
                          double *aa_src_or_wall, const double *uq, const double *tri_hmin, double tau_thr,
                          int use_hmin, double *const *mom_out, cudaStream_t s);
int launch_wall_trace(pbte_ctx *c, const double *vdf, const double *tri_fc_fc, int nk,
                      const int32_t *tri_list, const int32_t *lfc_list, double *out,
                      cudaStream_t s);
int launch_correct(pbte_ctx *c, double *vdf, const double *uq, const double *tri_hmin,
                   double tau_thr, int use_hmin, double *ts, double *qxs, double *qys,
                   double *temp, double *qx, double *qy, cudaStream_t s);
int launch_element_integrals(pbte_ctx *c, const double *ts, const double *qxs, const double *qys,
                             double *temp, double *qx, double *qy, cudaStream_t s);
int launch_batched_inverse(const double *a, double *inv, int n, int m, int32_t *singular,
                           cudaStream_t s);
// partner values of the periodic faces: mode 0 vdf -> compact [ndir][n_pfaces][nd]
// (gather), mode 1 compact -> full pbuf [ndir][n_faces][nd] rows (scatter)
int launch_periodic_copy(pbte_ctx *c, const double *src, double *dst, int mode, cudaStream_t s);
}  // namespace pbte

#define PBTE_CUDA_TRY(expr)                                  \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) return PBTE_ERR_CUDA;         \
    } while (0)
