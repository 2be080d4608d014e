// extern "C" entry points of libpbte_gb300: argument checks, then the
// launchers.  Every call is asynchronous on the caller's stream.
#include <cuda_runtime.h>

#include "pbte_internal.cuh"

namespace {
inline cudaStream_t S(void *s) { return reinterpret_cast<cudaStream_t>(s); }
}  // namespace

extern "C" {

const char *pbte_version(void) { return "pbte_gb300 1.0 (sm_103a)"; }

int pbte_sweep(pbte_ctx *c, const double *ts, const double *qxs, const double *qys, double *vdf,
               const double *flux_wall, const double *pbuf, int use_pbuf, void *stream) {
    if (!c || !ts || !qxs || !qys || !vdf) return PBTE_ERR_ARG;
    if (c->n_wall_ad && !flux_wall) return PBTE_ERR_ARG;
    if (use_pbuf && !pbuf) return PBTE_ERR_ARG;
    int rc = pbte::launch_sources(c, ts, qxs, qys, false, S(stream));
    if (rc) return rc;
    return pbte::launch_sweep64(c, vdf, flux_wall, pbuf, use_pbuf, S(stream));
}

int pbte_sweep_f32(pbte_ctx *c, const double *ts, const double *qxs, const double *qys, float *vdf32,
                   const double *flux_wall, double wall_scale, void *stream) {
    if (!c || !ts || !qxs || !qys || !vdf32) return PBTE_ERR_ARG;
    if (c->n_wall_ad && !flux_wall) return PBTE_ERR_ARG;
    if (c->has_periodic) return PBTE_ERR_UNSUPPORTED;
    int rc = pbte::launch_sources(c, ts, qxs, qys, true, S(stream));
    if (rc) return rc;
    return pbte::launch_sweep32(c, vdf32, flux_wall, wall_scale, S(stream));
}

int pbte_fixed_point_f32(pbte_ctx *c, const double *ts, const double *qxs, const double *qys,
                         const double *flux_wall_in, double wall_scale, float *vdf32, double *ts_out,
                         double *qxs_out, double *qys_out, double *flux_wall_out, double *temp, double *qx,
                         double *qy, void *stream) {
    if (!c || !ts || !qxs || !qys || !vdf32 || !ts_out || !qxs_out || !qys_out) return PBTE_ERR_ARG;
    if (c->n_wall_ad && (!flux_wall_in || !flux_wall_out)) return PBTE_ERR_ARG;
    if ((temp == nullptr) != (qx == nullptr) || (temp == nullptr) != (qy == nullptr)) return PBTE_ERR_ARG;
    if (c->has_periodic) return PBTE_ERR_UNSUPPORTED;
    return pbte::launch_fixed_point32(c, ts, qxs, qys, flux_wall_in, wall_scale, vdf32, ts_out, qxs_out, qys_out,
                                      flux_wall_out, temp, qx, qy, S(stream));
}

int pbte_moments(pbte_ctx *c, const double *vdf, double *ts, double *qxs, double *qys, double *temp,
                 double *qx, double *qy, void *stream) {
    if (!c || !vdf || !ts || !qxs || !qys) return PBTE_ERR_ARG;
    if ((temp == nullptr) != (qx == nullptr) || (temp == nullptr) != (qy == nullptr)) return PBTE_ERR_ARG;
    return pbte::launch_moments64(c, vdf, ts, qxs, qys, temp, qx, qy, S(stream));
}

int pbte_moments_f32(pbte_ctx *c, const float *vdf32, double *ts, double *qxs, double *qys, double *temp,
                     double *qx, double *qy, void *stream) {
    if (!c || !vdf32 || !ts || !qxs || !qys) return PBTE_ERR_ARG;
    if ((temp == nullptr) != (qx == nullptr) || (temp == nullptr) != (qy == nullptr)) return PBTE_ERR_ARG;
    return pbte::launch_moments32(c, vdf32, ts, qxs, qys, temp, qx, qy, S(stream));
}

int pbte_wall_flux(pbte_ctx *c, const double *vdf, double *flux_wall, void *stream) {
    if (!c || !vdf || (c->n_wall_ad && !flux_wall)) return PBTE_ERR_ARG;
    return pbte::launch_wall_flux64(c, vdf, flux_wall, S(stream));
}

int pbte_wall_flux_f32(pbte_ctx *c, const float *vdf32, double *flux_wall, void *stream) {
    if (!c || !vdf32 || (c->n_wall_ad && !flux_wall)) return PBTE_ERR_ARG;
    return pbte::launch_wall_flux32(c, vdf32, flux_wall, S(stream));
}

int pbte_residual_iterate(pbte_ctx *c, const double *temp, double *t_old, double *out, void *stream) {
    if (!c || !temp || !t_old || !out) return PBTE_ERR_ARG;
    return pbte::launch_residual(c, temp, t_old, out, S(stream));
}

int pbte_set_sweep_variant(pbte_ctx *c, int variant) {
    if (!c || variant < 0 || variant > 2) return PBTE_ERR_ARG;
    c->sweep_variant = variant;
    return PBTE_OK;
}

int pbte_set_ring_groups(pbte_ctx *c, int groups) {
    if (!c || groups < 0 || groups > 15) return PBTE_ERR_ARG;
    c->ring_groups = groups;
    return PBTE_OK;
}

int pbte_set_ring_width(pbte_ctx *c, int threads_per_group) {
    if (!c || (threads_per_group != 0 && threads_per_group != 64 && threads_per_group != 128)) return PBTE_ERR_ARG;
    c->ring_width = threads_per_group;
    return PBTE_OK;
}

int pbte_ctx_schedule(const pbte_ctx *c, int64_t *ring_w, int64_t *ring_r, int64_t *n_unique_dirs) {
    if (!c) return PBTE_ERR_ARG;
    if (ring_w) *ring_w = c->ring_W;
    if (ring_r) *ring_r = c->ring_R;
    if (n_unique_dirs) *n_unique_dirs = c->n_udir;
    return PBTE_OK;
}

int pbte_set_done_flag(pbte_ctx *c, const int32_t *done) {
    if (!c) return PBTE_ERR_ARG;
    c->done = done;
    return PBTE_OK;
}

int pbte_residual_check(pbte_ctx *c, const double *res, double tol, int64_t tmax, int32_t *done,
                        int64_t *count, double *hist, int64_t hist_cap, void *stream) {
    if (!c || !res || !done || !count || hist_cap < 0) return PBTE_ERR_ARG;
    return pbte::launch_residual_check(c, res, tol, tmax, done, count, hist, hist_cap, S(stream));
}

int pbte_transport_residual(pbte_ctx *c, const double *ts, const double *qxs, const double *qys,
                            const double *vdf, const double *flux_wall, const double *pbuf, double *num,
                            double *den, void *stream) {
    if (!c || !ts || !qxs || !qys || !vdf || !num || !den) return PBTE_ERR_ARG;
    if (c->n_wall_ad && !flux_wall) return PBTE_ERR_ARG;
    return pbte::launch_transport_residual(c, ts, qxs, qys, vdf, flux_wall, pbuf, num, den, S(stream));
}

int pbte_factorise_f32(pbte_ctx *c, void *stream) {
    if (!c) return PBTE_ERR_ARG;
    if (c->deg > 3) return PBTE_ERR_UNSUPPORTED;
    if (!c->d_lu32) {
        const size_t n = pbte::factor_count(c->n_udir, c->n_tris, c->nd * c->nd);
        if (cudaMalloc((void **)&c->d_lu32, n * sizeof(float)) != cudaSuccess) {
            c->d_lu32 = nullptr;
            return PBTE_ERR_NOMEM;
        }
        c->device_bytes += n * sizeof(float);
        pbte::g_live_bytes += (long long)(n * sizeof(float));
    }
    int rc = pbte::launch_factorise32(c, S(stream));
    if (rc) {
        cudaFree(c->d_lu32);
        c->d_lu32 = nullptr;
    }
    return rc;
}

int pbte_periodic_count(const pbte_ctx *c, int64_t *n_pfaces) {
    if (!c || !n_pfaces) return PBTE_ERR_ARG;
    *n_pfaces = c->n_pfaces;
    return PBTE_OK;
}

int pbte_periodic_gather(pbte_ctx *c, const double *vdf, double *out, void *stream) {
    if (!c || !vdf || (c->n_pfaces && !out)) return PBTE_ERR_ARG;
    return pbte::launch_periodic_copy(c, vdf, out, 0, S(stream));
}

int pbte_periodic_scatter(pbte_ctx *c, const double *in, double *pbuf, void *stream) {
    if (!c || (c->n_pfaces && (!in || !pbuf))) return PBTE_ERR_ARG;
    return pbte::launch_periodic_copy(c, in, pbuf, 1, S(stream));
}

int pbte_hot_source(pbte_ctx *c, const double *vdf, double tc5, double *work, void *stream) {
    if (!c || !vdf || !work) return PBTE_ERR_ARG;
    return pbte::launch_hot_source(c, vdf, tc5, work, S(stream));
}

int pbte_wall_trace(pbte_ctx *c, const double *vdf, const double *tri_fc_fc, int32_t nk, const int32_t *tri_list,
                    const int32_t *lfc_list, double *out, void *stream) {
    if (!c || !vdf || nk < 0 || (nk && (!tri_fc_fc || !tri_list || !lfc_list || !out))) return PBTE_ERR_ARG;
    return pbte::launch_wall_trace(c, vdf, tri_fc_fc, nk, tri_list, lfc_list, out, S(stream));
}

int pbte_correct(pbte_ctx *c, double *vdf, const double *uq, const double *tri_hmin, double tau_thr,
                 int use_hmin, double *ts, double *qxs, double *qys, double *temp, double *qx, double *qy,
                 void *stream) {
    if (!c || !vdf || !uq || !tri_hmin || !ts || !qxs || !qys || !temp || !qx || !qy) return PBTE_ERR_ARG;
    return pbte::launch_correct(c, vdf, uq, tri_hmin, tau_thr, use_hmin, ts, qxs, qys, temp, qx, qy, S(stream));
}

int pbte_gmres_columns_f32(pbte_ctx *c, const pbte_gmres_cycle_f32 *a, int32_t j0, int32_t j1, void *stream) {
    if (!c || !a || j0 < 0 || j1 <= j0 || j1 >= PBTE_MAX_BASIS || !a->Q || !a->uin || !a->uout || !a->w || !a->state) return PBTE_ERR_ARG;
    if (a->ldq < a->n || a->ldr < j1) return PBTE_ERR_ARG;
    if (!a->ts || !a->qxs || !a->qys || !a->vdf32 || !a->ts_out || !a->qxs_out || !a->qys_out) return PBTE_ERR_ARG;
    if (c->n_wall_ad && (!a->flux_wall_in || !a->flux_wall_out)) return PBTE_ERR_ARG;
    if ((a->temp == nullptr) != (a->qx == nullptr) || (a->temp == nullptr) != (a->qy == nullptr)) return PBTE_ERR_ARG;
    if (c->has_periodic) return PBTE_ERR_UNSUPPORTED;
    // the operator input is the state itself ([ts | qxs | qys | ...] = uin):
    // then the basis update can also form the next product's moment sources
    const int64_t k = (int64_t)c->nd * c->n_tris;
    const bool state_input = a->ts == a->uin && a->qxs == a->uin + k && a->qys == a->uin + 2 * k;
    const int32_t *before = c->done;
    c->done = a->state;
    int rc = PBTE_OK;
    // the basis update of column j also leaves column j+1's moment sources
    // (launch_next_basis_sources), so only a call's first product forms them
    bool have_sources = false;
    for (int32_t j = j0; j < j1 && rc == PBTE_OK; ++j) {
        rc = pbte::launch_fixed_point32(c, a->ts, a->qxs, a->qys, a->flux_wall_in, a->wall_scale, a->vdf32,
                                        a->ts_out, a->qxs_out, a->qys_out, a->flux_wall_out, a->temp, a->qx, a->qy,
                                        S(stream), !have_sources);
        if (rc == PBTE_OK)
            rc = pbte::arnoldi_column_givens_f32(a->Q, a->ldq, j + 1, a->uout, a->g, a->w, a->n, a->h, a->scratch,
                                                 a->scratch_len, a->R, a->ldr, a->cs, a->sn, a->gam, a->tol_abs,
                                                 a->state, a->hist, S(stream));
        if (rc == PBTE_OK) {
            const bool fuse = state_input;
            rc = fuse ? pbte::launch_next_basis_sources(c, j, a->w, a->h, a->Q, a->ldq, a->uin, a->n, a->state,
                                                        S(stream))
                      : PBTE_ERR_UNSUPPORTED;
            have_sources = rc == PBTE_OK;
            if (rc == PBTE_ERR_UNSUPPORTED)
                rc = pbte_gmres_next_basis_f32(j, a->w, a->h, a->Q, a->ldq, a->uin, a->n, a->state, stream);
        }
    }
    c->done = before;
    return rc;
}

int pbte_batched_inverse(const double *a, double *inv, int32_t n, int32_t m, int32_t *singular, void *stream) {
    if (!a || !inv || !singular || n < 0 || m <= 0) return PBTE_ERR_ARG;
    return pbte::launch_batched_inverse(a, inv, n, m, singular, S(stream));
}

}  // extern "C"
