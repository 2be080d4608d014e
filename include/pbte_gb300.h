/*
 * pbte_gb300.h -- C ABI of the GB300 (sm_103a) transport-sweep library.
 *
 * The library replaces the hot path of pybte's steady gray linearised-
 * Callaway DG discrete-ordinates solve (solver-python/pybte): the per-
 * direction upwind sweep, the angular moments, the adiabatic-wall emission,
 * the step and transport residuals, and the GSIS per-iteration kernels.
 * Each entry point names the reference function it stands in for.
 *
 * Conventions
 *  - Every function returns an int status: PBTE_OK (0), or a negative
 *    PBTE_ERR_* code.  No C++ exception crosses this boundary.
 *  - pbte_ctx_create takes HOST arrays (copied once); every other call takes
 *    DEVICE pointers (e.g. torch tensor data_ptr()) and a cudaStream_t passed
 *    as void*.  Calls are asynchronous on that stream.
 *  - Array layouts are the reference's (C order, 0-based):
 *      vdf[ndir][n_tris][ndof]      ts, qxs, qys[ndof][n_tris]
 *      temp, qx, qy[n_tris]         flux_wall[n_faces][ndof]
 *      pbuf[ndir][n_faces][ndof]
 *    Directions are flattened d = j1 + npole*j2 as in pybte/velocity.py:52-56.
 */
#ifndef PBTE_GB300_H
#define PBTE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBTE_OK 0
#define PBTE_ERR_ARG (-1)          /* bad argument / size                    */
#define PBTE_ERR_CUDA (-2)         /* a CUDA runtime call failed             */
#define PBTE_ERR_CYCLE (-3)        /* a direction's sweep graph has a cycle  */
#define PBTE_ERR_UNSUPPORTED (-4)  /* configuration not implemented          */
#define PBTE_ERR_TIMEOUT (-5)      /* a device-side wait ran out of its cap  */
#define PBTE_ERR_SINGULAR (-6)     /* singular element operator(s)           */
#define PBTE_ERR_NOMEM (-7)        /* device allocation failed               */

/* Krylov bases of the device GMRES hold at most PBTE_MAX_BASIS rows; a
 * pbte_cgs2 / pbte_arnoldi_column call over `rows` basis rows needs
 * PBTE_CGS2_SCRATCH_ROWS(rows) doubles of scratch (PBTE_CGS2_SCRATCH: up to
 * 64 rows). */
#define PBTE_MAX_BASIS 1024
#define PBTE_CGS2_SCRATCH_ROWS(rows) (8 + 2 * PBTE_MAX_BASIS + 1216 * ((((rows) + 7) / 8) * 8))
#define PBTE_CGS2_SCRATCH PBTE_CGS2_SCRATCH_ROWS(64)

/* precision of the sweep arithmetic */
#define PBTE_FP64 0
#define PBTE_FP32 1

typedef struct pbte_ctx pbte_ctx;

/* One case, host pointers, reference layouts.  The operator description is
 * the compact form of pybte's integral tensors (pybte/integration.py:159-404):
 *   mass[:,:,i] = area2[i] * ref_mass
 *   gx[i]       = area2[i] * (dxi[i][0] * ref_dx + dxi[i][1] * ref_dy)
 *   gy[i]       = area2[i] * (deta[i][0] * ref_dx + deta[i][1] * ref_dy)
 *   fcm[i][il]  = edge_scale[i][il] * ref_edge[il]
 *   ttfc[i][il] = fcm[i][il] gathered through edge_map[i][il][:]
 * with edge_dofs[il][:] the element DOFs on local edge il.             */
typedef struct {
    int32_t n_tris, n_faces, ndof, ndof_fc, ndir, nbc;
    double cv, vg, tau_r, tau_n, tau_c;
    const double *cxv, *cyv, *domega;          /* [ndir]                     */
    const double *ref_mass, *ref_dx, *ref_dy;  /* [ndof*ndof]                */
    const double *ref_edge;                    /* [3*ndof*ndof]              */
    const int32_t *edge_dofs;                  /* [3*ndof_fc]                */
    const double *area2;                       /* [n_tris]                   */
    const double *dxi, *deta;                  /* [n_tris*2]                 */
    const double *edge_scale;                  /* [n_tris*3]                 */
    const double *nx, *ny;                     /* [n_tris*3] outward normals */
    const int32_t *tri_faces;                  /* [n_tris*3]                 */
    const int32_t *upwind_tri;                 /* [n_tris*3] neighbour / periodic partner / -1 */
    const int32_t *edge_map;                   /* [n_tris*3*ndof_fc]         */
    const int32_t *face_bc;                    /* [n_faces]  -1 interior     */
    const int32_t *face_tri, *face_lfc;        /* [n_faces*2]                */
    const int32_t *bc_type;                    /* [nbc] 1 therm. 2 adiab. 3 periodic */
    const double *bc_temp;                     /* [nbc]                      */
    const double *int_tri;                     /* [ndof*n_tris]              */
} pbte_case_desc;

/* Build a sweep context: level schedules per direction class (host C++),
 * device copies of the compact operators, and -- when `precompute` is set --
 * the FP64 LU factors of every (direction, element) operator.
 * Replaces SweepContext.build + factorise (pybte/sweep.py:74-129).
 * Returns PBTE_ERR_CYCLE if a direction's sweep graph has a cycle, and
 * PBTE_ERR_SINGULAR if a precomputed factorisation meets a zero pivot. */
int pbte_ctx_create(const pbte_case_desc *desc, int precompute, pbte_ctx **out);
int pbte_ctx_destroy(pbte_ctx *ctx);

/* The direction classes pbte_ctx_create schedules with, host only (no GPU
 * needed): dir_class[ndir] receives each ordinate's class -- ordinates whose
 * c.n has the same sign on every interior and periodic face (seen from the
 * face's first side) share one level schedule -- numbered by first
 * appearance, *n_classes their count.  Reads the face arrays, normals and
 * ordinates of desc.  No reference counterpart (pybte orders each direction
 * on its own, pybte/ordering.py:61-140). */
int pbte_direction_classes(const pbte_case_desc *desc, int32_t *dir_class, int32_t *n_classes);

/* The wavefront level of every element for ordinate `dir`, host only: level
 * = 1 + the deepest element it waits for in the sweep (an interior upwind
 * neighbour, or a periodic partner that comes earlier in pybte's TRI_ORDER,
 * pybte/ordering.py:61-140), as pbte_ctx_create schedules the ordinate's
 * class; level[n_tris], *n_levels the count.  PBTE_ERR_CYCLE on a cycle. */
int pbte_direction_levels(const pbte_case_desc *desc, int32_t dir, int32_t *level, int32_t *n_levels);

/* Sweep kernel selection: 0 automatic (ring-pipelined when the level ring
 * fits in shared memory, else level-serial), 1 level-serial, 2 ring only
 * (PBTE_ERR_UNSUPPORTED from the sweep if it does not fit).  No reference
 * counterpart (pybte's mode switch is precomputed vs on-the-fly). */
int pbte_set_sweep_variant(pbte_ctx *ctx, int variant);

/* Shape of the ring sweep's blocks, the tuning knobs of the autotuner: the
 * pipeline depth (thread groups per block; 0 = default 4, at most 8 are
 * used) and the threads per group (0 = 64, or 64 or 128).  Shapes the
 * library has no kernel for on the mesh fall back to four groups of 64.  And
 * the schedule the context derived: widest level, deepest upwind level gap,
 * and the number of distinct in-plane velocities (one sweep block each).
 * No reference counterpart. */
int pbte_set_ring_groups(pbte_ctx *ctx, int groups);
int pbte_set_ring_width(pbte_ctx *ctx, int threads_per_group);
int pbte_ctx_schedule(const pbte_ctx *ctx, int64_t *ring_w, int64_t *ring_r,
                      int64_t *n_unique_dirs);

/* Sizes the context was built with, and the device bytes it holds. */
int pbte_ctx_info(const pbte_ctx *ctx, int64_t *n_levels_max, int64_t *n_classes,
                  int64_t *device_bytes);

/* Zero pivots met by the context's element factorisations so far (setup and
 * every on-the-fly sweep); reset != 0 sets the count back to zero.  pybte's
 * precomputed mode raises LinAlgError for these at setup (sweep.py:122-128);
 * in its on-the-fly mode a singular operator yields inf/NaN silently.
 * Synchronises with the device. */
int pbte_singular_count(pbte_ctx *ctx, int64_t *count, int reset);

/* Device bytes held by all live contexts of this process (the sum of their
 * pbte_ctx_info device_bytes).  No reference counterpart: a serving loop's
 * admission check, and evidence that failed context creation frees what it
 * allocated. */
int pbte_device_bytes_live(int64_t *bytes);

/* One FP64 transport sweep, in place on vdf.  Replaces SweepContext.sweep
 * (pybte/sweep.py:132-158 -> _kernels.sweep_precomputed/_onthefly,
 * pybte/_kernels.py:218-269).  `pbuf`/`use_pbuf` as in the reference
 * (_kernels.py:170-215): with use_pbuf every periodic face reads its
 * partner's row pbuf[d][face] (the Krylov path's explicit state); without,
 * a periodic face reads the partner's current vdf as the reference's
 * sequential sweep does -- this sweep's value when the partner comes first
 * in the direction's TRI_ORDER, else the previous sweep's.  pbuf may be
 * NULL when use_pbuf == 0. */
int pbte_sweep(pbte_ctx *ctx, const double *ts, const double *qxs, const double *qys,
               double *vdf, const double *flux_wall, const double *pbuf, int use_pbuf,
               void *stream);

/* Store FP32 element factors for the FP32 sweeps (P1-P3): one set per
 * distinct in-plane velocity, made with the FP32 sweep's own arithmetic, so
 * FP32 sweeps give the same bits with or without them; afterwards the FP32
 * sweeps load instead of assembling and factoring.  4 * ndof^2 bytes per
 * (element, distinct velocity).  No reference counterpart (FP32 path). */
int pbte_factorise_f32(pbte_ctx *ctx, void *stream);

/* Periodic faces of the context (faces with a periodic boundary, in
 * increasing face index) and their partner elements' DOFs, the periodic
 * block of the Krylov state (pybte/krylov.py:74-110):
 * pbte_periodic_gather: out[d][q][l] = vdf[d][partner(q)][l];
 * pbte_periodic_scatter: pbuf[d][face(q)][l] = in[d][q][l] (other rows of
 * pbuf untouched).  q < *n_pfaces. */
int pbte_periodic_count(const pbte_ctx *ctx, int64_t *n_pfaces);
int pbte_periodic_gather(pbte_ctx *ctx, const double *vdf, double *out, void *stream);
int pbte_periodic_scatter(pbte_ctx *ctx, const double *in, double *pbuf, void *stream);

/* FP32 sweep (mixed precision): moments and wall emission read in FP64,
 * element solves and vdf32 in FP32.  With `wall_scale` = 0 the thermalising
 * walls emit nothing (the homogeneous sweep of a defect correction).  No
 * reference counterpart: the reference is FP64 only. */
int pbte_sweep_f32(pbte_ctx *ctx, const double *ts, const double *qxs, const double *qys,
                   float *vdf32, const double *flux_wall, double wall_scale, void *stream);

/* The FP32 fixed-point product of the mixed path in one call: moment
 * sources, FP32 sweep, moments (and, when temp/qx/qy are given, the element
 * integrals) and the adiabatic-wall emission, from the state (ts, qxs, qys,
 * flux_wall_in) to (ts_out, qxs_out, qys_out, flux_wall_out) -- the map of
 * FixedPointOperator.apply (pybte/krylov.py:64-136) in FP32.  z-mirror
 * twins are folded (P1-P3, ring sweep): vdf32 is scratch whose first rows
 * hold one copy per distinct in-plane velocity, and the moments and the
 * emission read them with the pair's summed weight.  No reference
 * counterpart: the reference is FP64 only. */
int pbte_fixed_point_f32(pbte_ctx *ctx, const double *ts, const double *qxs, const double *qys,
                         const double *flux_wall_in, double wall_scale, float *vdf32, double *ts_out,
                         double *qxs_out, double *qys_out, double *flux_wall_out, double *temp,
                         double *qx, double *qy, void *stream);

/* Angular moments and element integrals.  Replaces compute_moments
 * (pybte/moments.py:51-55 -> _kernels.moments_kernel, _kernels.py:312-338).
 * temp, qx, qy may all be NULL to skip the element integrals.  The partial
 * sums go to scratch in the context: calls on one context must not overlap
 * on the GPU. */
int pbte_moments(pbte_ctx *ctx, const double *vdf, double *ts, double *qxs, double *qys,
                 double *temp, double *qx, double *qy, void *stream);
/* The same from an FP32 distribution, accumulated in FP32 per direction
 * block and summed in FP64. */
int pbte_moments_f32(pbte_ctx *ctx, const float *vdf32, double *ts, double *qxs, double *qys,
                     double *temp, double *qx, double *qy, void *stream);

/* Adiabatic-wall emission from vdf.  Replaces BoundaryData.update_wall_flux
 * (pybte/bc.py:47-58 -> _kernels.wall_flux_kernel, _kernels.py:364-397). */
int pbte_wall_flux(pbte_ctx *ctx, const double *vdf, double *flux_wall, void *stream);
int pbte_wall_flux_f32(pbte_ctx *ctx, const float *vdf32, double *flux_wall, void *stream);

/* Step residual sqrt(sum (T-T_old)^2 / sum T^2) into *out (device), then
 * t_old <- temp.  Replaces residual_iterate (pybte/moments.py:58-72). */
int pbte_residual_iterate(pbte_ctx *ctx, const double *temp, double *t_old, double *out,
                          void *stream);

/* Per-direction ||A f - b||^2_w numerator and denominator (device arrays of
 * ndir).  Replaces _kernels.transport_residual (pybte/_kernels.py:275-306),
 * the body of SweepContext.true_residual (pybte/sweep.py:161-197). */
int pbte_transport_residual(pbte_ctx *ctx, const double *ts, const double *qxs,
                            const double *qys, const double *vdf, const double *flux_wall,
                            const double *pbuf, double *num, double *den, void *stream);

/* The same transport residual for callers that cannot allocate device memory
 * where they call from (hosts whose device memory is handed out by their own
 * pool, where a cudaMalloc behind the pool's back fails or breaks its
 * accounting) or that must leave the context's scratch to a sweep in
 * flight.  It allocates nothing: the moment sources go to a static 4 MiB
 * device array (524288 doubles) held by every GPU that loads the library
 * until exit, so 3 * ndof * n_tris must be <= 524288 (else PBTE_ERR_ARG).
 * The first call on a device looks the array up (cudaGetSymbolAddress, with
 * that device current), which under lazy module loading is also when the
 * runtime commits the array's memory: make that first call before any
 * stream capture starts.  All calls
 * share the array, so calls that overlap on the GPU race; no state carries
 * from one call to the next.  Periodic faces: PBTE_ERR_UNSUPPORTED.  Call
 * it with the context's device current (the device current at
 * pbte_ctx_create): another device gives PBTE_ERR_ARG.
 * No counterpart in the reference. */
int pbte_transport_residual_noalloc(pbte_ctx *ctx, const double *ts, const double *qxs,
                                    const double *qys, const double *vdf,
                                    const double *flux_wall, double *num, double *den,
                                    void *stream);

/* Device-side stop flag for graph-captured iteration: when *done != 0 every
 * sweep/moment/residual kernel launched with the context returns at once.
 * pbte_set_done_flag(ctx, ptr) installs it (NULL removes it).
 * pbte_residual_check implements the source-iteration stopping rule of
 * pybte/driver.py:185-211 on the device: unless *done is already set it
 * records (res[0], res[1]) at hist[2*count] (when count < hist_cap),
 * increments *count, and sets *done = 1 if res[0] < tol, or *done = 2 if
 * *count reached tmax. */
int pbte_set_done_flag(pbte_ctx *ctx, const int32_t *done);
int pbte_residual_check(pbte_ctx *ctx, const double *res, double tol, int64_t tmax,
                        int32_t *done, int64_t *count, double *hist, int64_t hist_cap,
                        void *stream);

/* Classical Gram-Schmidt applied twice against the Krylov rows Q[0..rows-1]
 * (row stride ldq elements), in place on w, as in gmres_full
 * (pybte/krylov.py:201-210): h[0..rows-1] = c1 + c2 and h[rows] = ||w||.
 * Deterministic (block partial sums added in a fixed order).  `scratch`
 * holds scratch_len >= PBTE_CGS2_SCRATCH_ROWS(rows) doubles (PBTE_ERR_ARG
 * otherwise), all zero before its first use; a call leaves it ready for the
 * next one (for any row count), and concurrent calls need separate scratch.
 * rows <= PBTE_MAX_BASIS.  pbte_cgs2 keeps the basis and w in FP64; pbte_cgs2_f32 keeps
 * them in FP32 (FP32 products and warp sums, FP64 block and cross-block
 * sums; no reference counterpart: the inner solve of the mixed-precision
 * mode, whose operator is an FP32 sweep). */
int pbte_cgs2(const double *Q, int64_t ldq, int32_t rows, double *w, int64_t n, double *h,
              double *scratch, int64_t scratch_len, void *stream);
int pbte_cgs2_f32(const float *Q, int64_t ldq, int32_t rows, float *w, int64_t n, double *h,
                  double *scratch, int64_t scratch_len, void *stream);

/* One Arnoldi column after the product F(q_j) is in uout (the operator's
 * output, FP64, first n entries): w = q_j - (uout - g) with q_j = Q[rows-1]
 * (g may be NULL: w = q_j - uout), then the CGS2 of pbte_cgs2 /
 * pbte_cgs2_f32 -- gmres_full's product and orthogonalisation
 * (pybte/krylov.py:195-210) in three launches.  `done` (may be NULL): a
 * device flag; while it is nonzero every launch returns at once. */
int pbte_arnoldi_column(const double *Q, int64_t ldq, int32_t rows, const double *uout, const double *g,
                        double *w, int64_t n, double *h, double *scratch, int64_t scratch_len,
                        const int32_t *done, void *stream);
int pbte_arnoldi_column_f32(const float *Q, int64_t ldq, int32_t rows, const double *uout,
                            const double *g, float *w, int64_t n, double *h, double *scratch,
                            int64_t scratch_len, const int32_t *done, void *stream);

/* The host part of a GMRES column on the device, so that a restart cycle
 * runs as captured launches without a host round trip per column
 * (gmres_full, pybte/krylov.py:211-235): pbte_gmres_givens applies the
 * earlier rotations to the Hessenberg column h[0..j+1], forms rotation j
 * (hypot), stores column j of R at R[j*ldr + 0..j], updates the residual
 * estimates gam, writes hist[j] = |gam[j+1]| and the state: state[0] = 1
 * when |gam[j+1]| <= *tol_abs (a device scalar, so a captured cycle serves
 * any tolerance), 2 on breakdown (h[j+1] == 0); state[1] =
 * columns done.  pbte_gmres_next_basis(_f32) stores q_{j+1} = w / h[j+1] in
 * row j+1 of Q and widened into the operator input uin[0..n).  Both do
 * nothing while state[0] != 0; j + 1 < PBTE_MAX_BASIS.
 *
 * pbte_gmres_givens_bounded adds the stopping rule run_krylov wraps around
 * gmres_full (pybte/krylov.py:332-338): tol2 = [tol_abs, enough] and state
 * = [stop, columns, products before this cycle, reached (-1: none)].  The
 * first product (index n = state[2] + j + 1 among the run's products) whose
 * residual is <= enough sets state[3] = n; once n - state[3] > max(64,
 * state[3] / 4) the solve halts with state[0] = 3.  Precedence as
 * gmres_full: converged (1), halted (3), breakdown (2).
 * pbte_arnoldi_column_givens is pbte_arnoldi_column (FP64, done = state)
 * with that rotation (bounded != 0: the bounded form) run by the last block
 * of its norm pass. */
int pbte_gmres_givens(int32_t j, const double *h, double *R, int32_t ldr, double *cs, double *sn,
                      double *gam, const double *tol_abs, int32_t *state, double *hist, void *stream);
int pbte_gmres_givens_bounded(int32_t j, const double *h, double *R, int32_t ldr, double *cs, double *sn,
                              double *gam, const double *tol2, int32_t *state, double *hist, void *stream);
int pbte_arnoldi_column_givens(const double *Q, int64_t ldq, int32_t rows, const double *uout,
                               const double *g, double *w, int64_t n, double *h, double *scratch,
                               int64_t scratch_len, double *R, int32_t ldr, double *cs, double *sn,
                               double *gam, const double *tol2, int32_t *state, double *hist,
                               int32_t bounded, void *stream);
int pbte_gmres_next_basis(int32_t j, const double *w, const double *h, double *Q, int64_t ldq,
                          double *uin, int64_t n, const int32_t *state, void *stream);
int pbte_gmres_next_basis_f32(int32_t j, const float *w, const double *h, float *Q, int64_t ldq,
                              double *uin, int64_t n, const int32_t *state, void *stream);

/* Columns j0..j1-1 of a GMRES restart cycle with the FP32 fixed-point
 * product, issued from native code (one call records a whole chunk of a
 * captured cycle): per column the work of pbte_fixed_point_f32 on the
 * operator input, pbte_arnoldi_column_f32 (rows j+1, done = state),
 * pbte_gmres_givens and pbte_gmres_next_basis_f32 with their arithmetic,
 * with `state` installed as the context's stop flag for the duration
 * (pbte_set_done_flag); the rotation runs in the last block of the CGS2
 * norm pass -- the same numbers as those calls made one by one, in fewer
 * launches.  gmres_full's column loop
 * (pybte/krylov.py:190-240) for the mixed solver's inner GMRES.  The
 * operator views (ts/qxs/qys/flux_wall_in of the input uin, the outputs of
 * uout) are those pbte_fixed_point_f32 takes; flux_wall_in/out may be NULL
 * without adiabatic walls, temp/qx/qy may be NULL.  When ts/qxs/qys are the
 * first 3 * ndof * n_tris entries of uin in that order (the Krylov state),
 * the basis update of column j also forms column j+1's moment sources
 * (the same FP64 arithmetic), so only the call's first product launches
 * them.  0 <= j0 < j1, j1 + 1 <= rows of Q, j1 < PBTE_MAX_BASIS. */
typedef struct {
    const double *ts, *qxs, *qys, *flux_wall_in;   /* operator input: views of uin */
    double wall_scale;
    float *vdf32;                                  /* FP32 distribution scratch */
    double *ts_out, *qxs_out, *qys_out, *flux_wall_out, *temp, *qx, *qy;  /* views of uout */
    float *Q;                                      /* basis rows, leading dimension ldq */
    int64_t ldq;
    const double *uout, *g;                        /* g may be NULL */
    double *uin;
    float *w;
    int64_t n;
    double *h, *scratch;
    int64_t scratch_len;
    double *R;
    int32_t ldr;
    double *cs, *sn, *gam;
    const double *tol_abs;
    int32_t *state;
    double *hist;
} pbte_gmres_cycle_f32;
int pbte_gmres_columns_f32(pbte_ctx *ctx, const pbte_gmres_cycle_f32 *cyc, int32_t j0, int32_t j1,
                           void *stream);

/* GSIS per-iteration kernels (pybte/acceleration/):
 * third-order moment source, hot_source.py:29-58 -> work[n_tris][7*ndof];
 * kinetic wall-trace moments, global_solve.py:31-53 -> out[nk][3*ndof_fc];
 * damped correction, correction.py:29-75 (in place on vdf and moments). */
int pbte_hot_source(pbte_ctx *ctx, const double *vdf, double tc5, double *work, void *stream);
int pbte_wall_trace(pbte_ctx *ctx, const double *vdf, const double *tri_fc_fc, int32_t nk,
                    const int32_t *tri_list, const int32_t *lfc_list, double *out, void *stream);
int pbte_correct(pbte_ctx *ctx, double *vdf, const double *uq, const double *tri_hmin,
                 double tau_thr, int use_hmin, double *ts, double *qxs, double *qys,
                 double *temp, double *qx, double *qy, void *stream);

/* GSIS static condensation per iteration, on operator layouts made once at
 * setup (pbte_gb300/gsis.py), field-major so that consecutive threads read
 * consecutive addresses.  M = 7*ndof local unknowns per element, NF3 =
 * 3*ndof_fc trace unknowns per face.
 *   inv_t[(q*n_tris + i)*M + p]           = inv(AA_SOL_i)[p][q]
 *                                           (assembly.py:100, build_local_operators)
 *   ba1_t[(p*n_faces + f)*NF3 + r]        = BA_SOL[tri1[f], lfc][r][p] (assembly.py:128-184)
 *   ba2_t[(p*n2 + k)*NF3 + r]             = the same for the second element of the
 *                                           faces with slot2[f] = k >= 0 (tri2[k];
 *                                           mirror2[k] != 0: a periodic pair walked the
 *                                           same way, rows reversed within each block of
 *                                           ndof_fc, global_solve.py:151-157)
 *   aa_trace_t[((il*NF3 + r)*n_tris + i)*M + p] = AA_TRACE_i[il][p][r]
 *   wall_slot[f]: row of the kinetic wall moments (pbte_wall_trace output) or -1;
 *   wall_kind[f]: 1 thermalising, 2 diffuse adiabatic; wall_nx/ny: the wall
 *   element's outward normal on the face.  variant: 0 = A, 1 = B. */
typedef struct pbte_gsis_ops {
    int32_t n_tris, n_faces, ndof, ndof_fc, variant, n2, n_walls, pad;
    double cv;
    const double *inv_t;
    const double *ba1_t;
    const int32_t *tri1;
    const double *ba2_t;
    const int32_t *slot2;
    const int32_t *tri2;
    const int32_t *mirror2;
    const int32_t *wall_slot;
    const int32_t *wall_kind;
    const double *wall_nx, *wall_ny;
    const double *aa_trace_t;
    const int32_t *tri_faces;
} pbte_gsis_ops;

/* hot_source (acceleration/hot_source.py:29-75) including its inv_aa_sol @ work:
 * aa_src[i][p] (n_tris x 7*ndof) from the distribution.  The context's
 * stop flag (pbte_set_done_flag) makes it return at once. */
int pbte_gsis_hot_apply(pbte_ctx *ctx, const pbte_gsis_ops *ops, const double *vdf, double tc5,
                        double *aa_src, void *stream);
/* aa_src[i][p] = sum_{q=c0}^{c1-1} inv(AA_SOL_i)[p][q] work[i][q]: the element
 * solve of any local source (the moment preconditioner, krylov.py:369-414). */
int pbte_gsis_apply_inverse(const pbte_gsis_ops *ops, const double *work, int32_t c0, int32_t c1,
                            double *aa_src, const int32_t *done, void *stream);
/* GlobalSolver.rhs (acceleration/global_solve.py:131-187): ffa[f][r]
 * (n_faces x NF3, the solve's unknown order) from aa_src and the kinetic wall
 * moments.  done (optional device flag): return at once while *done != 0. */
int pbte_gsis_trace_rhs(const pbte_gsis_ops *ops, const double *aa_src, const double *wall_mom, double *ffa,
                        const int32_t *done, void *stream);
/* local_solve (acceleration/local_solve.py:16-26): uq[p][i] (7*ndof x n_tris) =
 * aa_src[i][p] + sum_il AA_TRACE_i[il] u_trace[face(i, il)]. */
int pbte_gsis_local_recover(const pbte_gsis_ops *ops, const double *aa_src, const double *u_trace, double *uq,
                            const int32_t *done, void *stream);

/* ---- many cases' folded FP32 sweeps in one launch per DG order ----------
 * (no reference counterpart: pybte solves one case at a time; the batched
 * solves of many uneven cases).  A batch is made once for a fixed set of
 * cases and buffers; each run launches, per case, the moment sources of its
 * ts/qxs/qys (when with_sources != 0; the context's stop flag applies), then
 * ONE ring-sweep kernel per DG order present, whose blocks are the distinct
 * velocities of all that order's cases: each block sweeps one velocity of
 * one case, exactly as pbte_sweep_fold_f32 does it alone (same arithmetic,
 * same results).  A case whose `done` flag (device int, may be NULL) is
 * nonzero is skipped.  groups x width is the block shape (thread groups of
 * 64 or 128 threads, 1 to 8 groups; P3 uses groups of 64, at most 4): the
 * autotuner's knob.  All cases on one device, no periodic faces, P1-P3.
 * Creating a batch allocates its case table on the device; runs allocate
 * nothing. */
typedef struct pbte_sweep_batch pbte_sweep_batch;
typedef struct {
    pbte_ctx *ctx;
    const double *ts, *qxs, *qys, *flux_wall;   /* flux_wall may be NULL without adiabatic walls */
    double wall_scale;
    float *vdf32;                               /* folded rows: [n_udir][n_tris][ndof] */
    const int32_t *done;
} pbte_batch_item;
int pbte_sweep_batch_create(int32_t n, const pbte_batch_item *items, int32_t groups, int32_t width,
                            pbte_sweep_batch **out);
int pbte_sweep_batch_run(pbte_sweep_batch *batch, int with_sources, void *stream);
int pbte_sweep_batch_destroy(pbte_sweep_batch *batch);

/* The FP32 GSIS product of the mixed-precision GSIS solve (no reference
 * counterpart: the inner operator of an FP64 defect correction around
 * Acceleration.apply, acceleration/__init__.py:95-115).  The distribution
 * is folded, vdf32[n_udir][n_tris][ndof]: one row per distinct in-plane
 * velocity (an ordinate and its z-mirror twin see the same transport, so
 * the pair is solved once and its weights summed).  No periodic faces; ndof
 * 3, 6 or 10 (PBTE_ERR_UNSUPPORTED otherwise).
 *  pbte_sweep_fold_f32: the moment sources of ts/qxs/qys and one FP32 sweep
 *    (pbte_sweep_f32's arithmetic) into the folded rows;
 *  pbte_fold_epilogue_f32: moments, element integrals (temp/qx/qy, all NULL
 *    or none) and the adiabatic wall emission (flux_wall, may be NULL) of a
 *    folded distribution;
 *  pbte_gsis_hot_apply_f32, pbte_wall_trace_f32, pbte_correct_f32: the hot
 *    source with the element inverses, the kinetic wall traces and the
 *    damped correction (pbte_correct: the distribution updated in place and
 *    the new moments ts/qxs/qys = the distribution's plus the damped
 *    corrections, all three NULL to skip; no element integrals) on the
 *    folded distribution, with FP32 angular sums. */
int pbte_sweep_fold_f32(pbte_ctx *ctx, const double *ts, const double *qxs, const double *qys,
                        const double *flux_wall, double wall_scale, float *vdf32, void *stream);
int pbte_fold_epilogue_f32(pbte_ctx *ctx, const float *vdf32, double *ts, double *qxs, double *qys,
                           double *flux_wall, double *temp, double *qx, double *qy, void *stream);
int pbte_gsis_hot_apply_f32(pbte_ctx *ctx, const pbte_gsis_ops *ops, const float *vdf32, double tc5,
                            double *aa_src, void *stream);
int pbte_wall_trace_f32(pbte_ctx *ctx, const float *vdf32, const double *tri_fc_fc, int32_t nk,
                        const int32_t *tri_list, const int32_t *lfc_list, double *out, void *stream);
int pbte_correct_f32(pbte_ctx *ctx, float *vdf32, const double *uq, const double *tri_hmin, double tau_thr,
                     int use_hmin, double *ts, double *qxs, double *qys, void *stream);

/* Batched dense inverse of n matrices of order m (FP64, Gauss-Jordan with
 * partial pivoting), a[n][m][m] -> inv[n][m][m].  Replaces the
 * np.linalg.inv of build_local_operators (acceleration/assembly.py:100).
 * *singular (device int) counts zero pivots. */
int pbte_batched_inverse(const double *a, double *inv, int32_t n, int32_t m, int32_t *singular,
                         void *stream);

/* ---- GSIS trace solve (pybte/acceleration/global_solve.py:120-195) --------
 * One height of the forward / backward sweep of a nested-dissection
 * multifrontal solve of K x = b (factors made once on the host,
 * pbte_gb300/trace_nd.py).  items: [n_items][4] int32 (node, first row,
 * end row, column groups kc: a power of two up to 64; at most 256 / kc
 * rows);
 * meta: [nodes][8] int64 (index offset, own count o, front size m, G
 * offset, H offset, delta offset, contribution-pointer offset, 0); idx: the
 * global unknowns of each front, own first; G: per node m x o, H: o x m,
 * both column-major; cptr/csrc: per front position, the delta slots of the
 * children's updates to add.  max_own / max_front: the largest o of the
 * forward items / m of the backward items (shared memory, at most 25 600
 * doubles).  done (optional device flag):
 * every block returns at once while *done != 0. */
int pbte_nd_forward(const int32_t *items, int32_t n_items, const int64_t *meta, const int32_t *idx,
                    const int64_t *cptr, const int64_t *csrc, const double *G, const double *b, double *z,
                    double *delta, int32_t max_own, const int32_t *done, void *stream);
int pbte_nd_backward(const int32_t *items, int32_t n_items, const int64_t *meta, const int32_t *idx,
                     const double *H, const double *z, double *x, int32_t max_front, const int32_t *done,
                     void *stream);

/* ---- field output (pybte/io_output.py:187-276) ---------------------------
 * No context: these take the mesh, basis and state as plain device arrays,
 * so they serve any solver's vdf.
 *
 * Angular moments per element DOF, the einsums of sample_fields
 * (io_output.py:235-237): m[l*n_tris + i] = sum_d w[d] * vdf[d][i][l] for the
 * weights w0 = domega, wx = cx*domega, wy = cy*domega. */
int pbte_field_moments(const double *vdf, int32_t ndir, int32_t n_tris, int32_t ndof, const double *w0,
                       const double *wx, const double *wy, double *m0, double *mx, double *my,
                       void *stream);

/* locate_points (io_output.py:187-217): out[i*ny + j] = the first element
 * (lowest index) whose three sub-areas at (px[i], py[j]) are all >= -1e-12,
 * or -1.  tri_x/tri_y: [n_tris][3] vertex coordinates.  The candidates come
 * from an nbx x nby bin grid (origin x0, y0; bin sizes hx, hy): bin
 * b = bx*nby + by lists bin_items[bin_start[b] .. bin_start[b+1]) in
 * increasing element index; the bin of a coordinate v is
 * clamp(floor((v - v0) / h), 0, nb - 1) and every element must be listed in
 * each bin its box, widened past the -1e-12 slack, touches.  One bin holding
 * every element is a plain scan. */
int pbte_locate_points(const double *tri_x, const double *tri_y, int32_t n_tris, double x0, double y0,
                       double hx, double hy, int32_t nbx, int32_t nby, const int32_t *bin_start,
                       const int32_t *bin_items, const double *px, int32_t nx, const double *py,
                       int32_t ny, int32_t *out, void *stream);

/* sample_fields (io_output.py:220-276): T = (phi . m0) / cv, qx = phi . mx,
 * qy = phi . my at every located point, and with uq (the GSIS macroscopic
 * unknowns [7*ndof][n_tris], or NULL for zeros) the stress trio
 * Nxx, Nxy, Nyy.  nodfun [ndof][ndof] and mono [ndof][2] are the basis's
 * monomial coefficients and exponents.  out: [6][nx*ny] in the order
 * T, qx, qy, Nxx, Nxy, Nyy; points with triid < 0 get zeros. */
int pbte_sample_fields(const double *tri_x, const double *tri_y, const int32_t *triid, const double *px,
                       int32_t nx, const double *py, int32_t ny, const double *nodfun, const int32_t *mono,
                       int32_t ndof, const double *m0, const double *mx, const double *my, int32_t n_tris,
                       double cv, const double *uq, double *out, void *stream);

/* Version string of the built library. */
const char *pbte_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PBTE_GB300_H */
