/*
 * pbte_oracle.c -- TEST INFRASTRUCTURE ONLY.  A plain-C restatement of the
 * reference's CPU kernels (dingtao-shen/...-PBTE, solver-python/pybte), used
 * as the parity checker for the GPU path and as the timed CPU baseline.  It
 * is never linked into, called by, or shipped with the product library.
 *
 * Every function follows one reference function statement for statement,
 * with the same floating-point operation order, so that (built with
 * -ffp-contract=off) it reproduces the reference's numpy/LAPACK path bit for
 * bit.  Array layouts are the reference's (C order, 0-based):
 *   order[ndir][n_tris]           mass[nd][nd][n_tris]  (M, L, I)
 *   gx, gy[n_tris][nd][nd]        fcm, ttfc[n_tris][3][nd][nd]
 *   nx, ny, tri_faces, neighbour[n_tris][3]
 *   face_bc, periodic_tri[n_faces]  bc_type, bc_temp[nbc]
 *   flux_wall[n_faces][nd]        vdf[ndir][n_tris][nd]
 *   ts, qxs, qys[nd][n_tris]      pbuf[ndir][n_faces][nd]
 * Directions are independent, so loops over them may run on OpenMP threads
 * without changing any result.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int ndir, n_tris, nd, n_faces, nbc;
    const int *order;
    const double *cxv, *cyv, *domega;
    double cv, vg, tau_r, tau_n, tau_c, pi;
    const double *mass, *gx, *gy, *fcm, *ttfc, *nx, *ny;
    const int *tri_faces, *face_bc, *neighbour, *periodic_tri, *bc_type;
    const double *bc_temp;
    const double *flux_wall;
} orc_ctx;

#define MAXND 16

/* DGETF2 look-alike: pybte/_kernels.py:44-76 (first max |a| pivot,
 * multipliers a * (1/pivot), fused rank-1 update).  Returns INFO. */
int orc_lu_factor(double *a, int *ipiv, int n)
{
    int info = 0;
    for (int k = 0; k < n; ++k) {
        int p = k;
        double big = fabs(a[k * n + k]);
        for (int i = k + 1; i < n; ++i) {
            double v = fabs(a[i * n + k]);
            if (v > big) { big = v; p = i; }
        }
        ipiv[k] = p;
        if (a[p * n + k] == 0.0) {
            if (info == 0) info = k + 1;
            continue;
        }
        if (p != k)
            for (int j = 0; j < n; ++j) {
                double t = a[k * n + j]; a[k * n + j] = a[p * n + j]; a[p * n + j] = t;
            }
        double r = 1.0 / a[k * n + k];
        for (int i = k + 1; i < n; ++i) a[i * n + k] = a[i * n + k] * r;
        for (int i = k + 1; i < n; ++i) {
            double aik = a[i * n + k];
            if (aik != 0.0)
                for (int j = k + 1; j < n; ++j) a[i * n + j] -= aik * a[k * n + j];
        }
    }
    return info;
}

/* DGETRS('N') look-alike for one right-hand side: pybte/_kernels.py:79-101
 * (back substitution with the column index descending). */
void orc_lu_solve(const double *a, const int *ipiv, double *b, int n)
{
    for (int k = 0; k < n; ++k) {
        int p = ipiv[k];
        if (p != k) { double t = b[k]; b[k] = b[p]; b[p] = t; }
    }
    for (int k = 0; k < n; ++k) {
        double bk = b[k];
        if (bk != 0.0)
            for (int i = k + 1; i < n; ++i) b[i] -= bk * a[i * n + k];
    }
    for (int k = n - 1; k >= 0; --k) {
        b[k] = b[k] / a[k * n + k];
        double bk = b[k];
        if (bk != 0.0)
            for (int i = 0; i < k; ++i) b[i] -= bk * a[i * n + k];
    }
}

/* A_SOL for element i, one direction: pybte/_kernels.py:107-125. */
static void fill_a_sol(const orc_ctx *c, double *a, int i, double cxd, double cyd, double inv_tau_c)
{
    const int nd = c->nd, nt = c->n_tris;
    double s0 = cxd * c->nx[i * 3 + 0] + cyd * c->ny[i * 3 + 0];
    double s1 = cxd * c->nx[i * 3 + 1] + cyd * c->ny[i * 3 + 1];
    double s2 = cxd * c->nx[i * 3 + 2] + cyd * c->ny[i * 3 + 2];
    double w0 = 0.5 * (s0 + fabs(s0));
    double w1 = 0.5 * (s1 + fabs(s1));
    double w2 = 0.5 * (s2 + fabs(s2));
    const double *gx = c->gx + (size_t)i * nd * nd, *gy = c->gy + (size_t)i * nd * nd;
    const double *f0 = c->fcm + ((size_t)i * 3 + 0) * nd * nd;
    const double *f1 = c->fcm + ((size_t)i * 3 + 1) * nd * nd;
    const double *f2 = c->fcm + ((size_t)i * 3 + 2) * nd * nd;
    for (int l = 0; l < nd; ++l)
        for (int m = 0; m < nd; ++m) {
            double v = (inv_tau_c * c->mass[((size_t)m * nd + l) * nt + i]
                        - cxd * gx[m * nd + l] - cyd * gy[m * nd + l]);
            v = v + w0 * f0[m * nd + l];
            v = v + w1 * f1[m * nd + l];
            v = v + w2 * f2[m * nd + l];
            a[m * nd + l] = v;
        }
}

/* Callaway source, the reference's expression order: pybte/_kernels.py:154-167. */
static void fill_a_src(const orc_ctx *c, double *src, int i, double cxd, double cyd,
                       const double *ts, const double *qxs, const double *qys)
{
    const int nd = c->nd, nt = c->n_tris;
    const double cv = c->cv, vg = c->vg, tau_r = c->tau_r, tau_n = c->tau_n, pi = c->pi;
    for (int m = 0; m < nd; ++m) {
        double acc = 0.0;
        for (int l = 0; l < nd; ++l) {
            double mlm = c->mass[((size_t)l * nd + m) * nt + i];
            double tl = ts[(size_t)l * nt + i];
            acc = acc + cv * tl / 4.0 / pi / tau_r * mlm;
            acc = acc + 1.0 / tau_n * mlm * (cv * tl / 4.0 / pi
                  + 3.0 / 4.0 / pi * (qxs[(size_t)l * nt + i] * cxd + qys[(size_t)l * nt + i] * cyd) / vg / vg);
        }
        src[m] = acc;
    }
}

/* Upwind inflow with the wall dispatch: pybte/_kernels.py:170-215. */
static void add_face_sources(const orc_ctx *c, double *src, int i, int d, double cxd, double cyd,
                             const double *vdf, const double *pbuf, int use_pbuf)
{
    const int nd = c->nd, nt = c->n_tris;
    for (int il = 0; il < 3; ++il) {
        double speed = cxd * c->nx[i * 3 + il] + cyd * c->ny[i * 3 + il];
        double w = 0.5 * (speed - fabs(speed));
        if (w == 0.0) continue;
        int fc = c->tri_faces[i * 3 + il];
        int bc = c->face_bc[fc];
        const double *tt = c->ttfc + ((size_t)i * 3 + il) * nd * nd;
        if (bc < 0) {
            int iext = c->neighbour[i * 3 + il];
            for (int l = 0; l < nd; ++l) {
                double fl = vdf[((size_t)d * nt + iext) * nd + l];
                for (int m = 0; m < nd; ++m) src[m] -= (w * tt[m * nd + l]) * fl;
            }
        } else {
            int typ = c->bc_type[bc];
            if (typ == 3) {
                int iext = c->periodic_tri[fc];
                for (int l = 0; l < nd; ++l) {
                    double fl = use_pbuf ? pbuf[((size_t)d * c->n_faces + fc) * nd + l]
                                         : vdf[((size_t)d * nt + iext) * nd + l];
                    for (int m = 0; m < nd; ++m) src[m] -= (w * tt[m * nd + l]) * fl;
                }
            } else if (typ == 2) {
                for (int m = 0; m < nd; ++m) src[m] -= w * (-c->flux_wall[(size_t)fc * nd + m]);
            } else {
                double tw = c->cv / 4.0 / c->pi * c->bc_temp[bc];
                for (int m = 0; m < nd; ++m) src[m] -= w * (tw * tt[m * nd + 0]);
            }
        }
    }
}

/* One transport sweep, factorising on the fly: pybte/_kernels.py:242-269
 * (identical in every bit to the precomputed variant, :218-239).
 * Returns the number of singular element operators met. */
int orc_sweep(const orc_ctx *c, const double *ts, const double *qxs, const double *qys,
              double *vdf, const double *pbuf, int use_pbuf, int nthreads)
{
    const int nd = c->nd, nt = c->n_tris;
    const double inv_tau_c = 1.0 / c->tau_c;
    int bad = 0;
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : bad) num_threads(nthreads > 0 ? nthreads : 1)
    for (int d = 0; d < c->ndir; ++d) {
        double a[MAXND * MAXND], src[MAXND];
        int p[MAXND];
        double cxd = c->cxv[d], cyd = c->cyv[d];
        for (int k = 0; k < nt; ++k) {
            int i = c->order[(size_t)d * nt + k];
            fill_a_sol(c, a, i, cxd, cyd, inv_tau_c);
            fill_a_src(c, src, i, cxd, cyd, ts, qxs, qys);
            add_face_sources(c, src, i, d, cxd, cyd, vdf, pbuf, use_pbuf);
            if (orc_lu_factor(a, p, nd)) bad += 1;
            orc_lu_solve(a, p, src, nd);
            for (int m = 0; m < nd; ++m) vdf[((size_t)d * nt + i) * nd + m] = src[m];
        }
    }
    return bad;
}

/* ||A f - b||^2 per direction, no sweep: pybte/_kernels.py:275-306. */
void orc_transport_residual(const orc_ctx *c, const double *ts, const double *qxs, const double *qys,
                            const double *vdf, const double *pbuf, double *out_num, double *out_den,
                            int nthreads)
{
    const int nd = c->nd, nt = c->n_tris;
    const double inv_tau_c = 1.0 / c->tau_c;
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (int d = 0; d < c->ndir; ++d) {
        double a[MAXND * MAXND], src[MAXND];
        double num = 0.0, den = 0.0;
        double cxd = c->cxv[d], cyd = c->cyv[d];
        for (int i = 0; i < nt; ++i) {
            fill_a_sol(c, a, i, cxd, cyd, inv_tau_c);
            fill_a_src(c, src, i, cxd, cyd, ts, qxs, qys);
            add_face_sources(c, src, i, d, cxd, cyd, vdf, pbuf, 0);
            for (int m = 0; m < nd; ++m) {
                double r = -src[m];
                for (int l = 0; l < nd; ++l) r += a[m * nd + l] * vdf[((size_t)d * nt + i) * nd + l];
                num += r * r * c->domega[d];
                den += src[m] * src[m] * c->domega[d];
            }
        }
        out_num[d] = num;
        out_den[d] = den;
    }
}

/* Calculate_Macro_Properties: pybte/_kernels.py:312-338. */
void orc_moments(int ndir, int nt, int nd, const double *vdf, const double *cxv, const double *cyv,
                 const double *domega, const double *int_tri, double cv, double *ts, double *qxs,
                 double *qys, double *temp, double *qx, double *qy)
{
    for (int i = 0; i < nt; ++i) { temp[i] = 0.0; qx[i] = 0.0; qy[i] = 0.0; }
    for (int i = 0; i < nt; ++i)
        for (int l = 0; l < nd; ++l) {
            double ss = 0.0, ssx = 0.0, ssy = 0.0;
            for (int d = 0; d < ndir; ++d) {
                double f = vdf[((size_t)d * nt + i) * nd + l];
                ss += f * domega[d];
                ssx += cxv[d] * f * domega[d];
                ssy += cyv[d] * f * domega[d];
            }
            ts[(size_t)l * nt + i] = ss / cv;
            qxs[(size_t)l * nt + i] = ssx;
            qys[(size_t)l * nt + i] = ssy;
            temp[i] += ss * int_tri[(size_t)l * nt + i] / cv;
            qx[i] += ssx * int_tri[(size_t)l * nt + i];
            qy[i] += ssy * int_tri[(size_t)l * nt + i];
        }
}

/* Sequential sums: pybte/_kernels.py:341-361. */
double orc_sum(const double *a, int n)
{
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += a[i];
    return s;
}

double orc_residual(const double *temp, const double *t_old, int n)
{
    double s1 = 0.0, s2 = 0.0;
    for (int i = 0; i < n; ++i) {
        double d = temp[i] - t_old[i];
        s1 += d * d;
        s2 += temp[i] * temp[i];
    }
    return sqrt(s1 / s2);
}

/* Diffuse adiabatic-wall emission: pybte/_kernels.py:364-397. */
void orc_wall_flux(int ndir, int nt, int nd, int n_faces, const double *vdf, const double *cxv,
                   const double *cyv, const double *domega, const double *fcm, const double *nx,
                   const double *ny, const int *face_bc, const int *face_tri, const int *face_lfc,
                   const int *bc_type, double *flux_wall)
{
    for (int f = 0; f < n_faces; ++f) {
        int bc = face_bc[f];
        if (bc < 0 || bc_type[bc] != 2) continue;
        int tri, lfc;
        if (face_tri[f * 2 + 0] < 0) { tri = face_tri[f * 2 + 1]; lfc = face_lfc[f * 2 + 1]; }
        else { tri = face_tri[f * 2 + 0]; lfc = face_lfc[f * 2 + 0]; }
        double n1 = -nx[tri * 3 + lfc], n2 = -ny[tri * 3 + lfc];
        const double *fm = fcm + ((size_t)tri * 3 + lfc) * nd * nd;
        for (int m = 0; m < nd; ++m) {
            double ss1 = 0.0, ss2 = 0.0;
            for (int d = 0; d < ndir; ++d) {
                double u = cxv[d] * n1 + cyv[d] * n2;
                if (u < 0.0) {
                    double acc = 0.0;
                    for (int l = 0; l < nd; ++l) acc += vdf[((size_t)d * nt + tri) * nd + l] * fm[m * nd + l];
                    ss1 += u * domega[d] * acc;
                } else {
                    ss2 -= u * domega[d];
                }
            }
            flux_wall[(size_t)f * nd + m] = -ss1 / ss2;
        }
    }
}

/* Per-direction topological order, ascending-index rescans, optional cycle
 * breaking: pybte/ordering.py:61-140.  Returns 0, or -1 on an unbroken cycle. */
int orc_order(int ndir, int nt, const int *neighbour, const double *nx, const double *ny,
              const double *cx, const double *cy, int *order, int *cycles, int allow_break)
{
    int status = 0;
    signed char *io = (signed char *)malloc((size_t)nt * 3);
    unsigned char *in = (unsigned char *)malloc((size_t)nt);
    for (int d = 0; d < ndir && status == 0; ++d) {
        memset(io, 0, (size_t)nt * 3);
        memset(in, 1, (size_t)nt);
        for (int i = 0; i < nt; ++i)
            for (int il = 0; il < 3; ++il)
                if (neighbour[i * 3 + il] >= 0) {
                    double flux = cx[d] * nx[i * 3 + il] + cy[d] * ny[i * 3 + il];
                    io[i * 3 + il] = flux > 0.0 ? 1 : (flux < 0.0 ? -1 : 0);
                }
        int num = 0, broken = 0;
        while (num < nt) {
            int progressed = 0;
            for (int i = 0; i < nt; ++i) {
                if (!in[i]) continue;
                if (io[i * 3] == -1 || io[i * 3 + 1] == -1 || io[i * 3 + 2] == -1) continue;
                order[(size_t)d * nt + num++] = i;
                in[i] = 0;
                progressed = 1;
                for (int il = 0; il < 3; ++il) {
                    int t2 = neighbour[i * 3 + il];
                    if (t2 >= 0)
                        for (int k = 0; k < 3; ++k)
                            if (neighbour[t2 * 3 + k] == i) { io[t2 * 3 + k] = 0; break; }
                }
            }
            if (!progressed) {
                if (!allow_break) { status = -1; break; }
                int best = -1, best_in = 4;
                for (int i = 0; i < nt; ++i) {
                    if (!in[i]) continue;
                    int cnt = (io[i * 3] == -1) + (io[i * 3 + 1] == -1) + (io[i * 3 + 2] == -1);
                    if (cnt < best_in) { best_in = cnt; best = i; }
                }
                if (best < 0) { status = -1; break; }
                order[(size_t)d * nt + num++] = best;
                in[best] = 0;
                broken++;
                for (int il = 0; il < 3; ++il) {
                    int t2 = neighbour[best * 3 + il];
                    if (t2 >= 0)
                        for (int k = 0; k < 3; ++k)
                            if (neighbour[t2 * 3 + k] == best) { io[t2 * 3 + k] = 0; break; }
                }
            }
        }
        cycles[d] = broken;
    }
    free(io);
    free(in);
    return status;
}

/* GSIS third-order moment source: pybte/acceleration/hot_source.py:29-58.
 * out[n_tris][7*nd], stress blocks only. */
void orc_hot_kernel(int ndir, int nt, int nd, const double *vdf, const double *gx, const double *gy,
                    const double *cxv, const double *cyv, const double *domega, double tc5, double *out)
{
    for (int i = 0; i < nt; ++i)
        for (int m = 0; m < nd; ++m) {
            double pixx = 0.0, pixy = 0.0, piyy = 0.0;
            for (int d = 0; d < ndir; ++d) {
                double cx = cxv[d], cy = cyv[d], dw = domega[d];
                double t = 0.0;
                for (int l = 0; l < nd; ++l) t += vdf[((size_t)d * nt + i) * nd + l] * gx[((size_t)i * nd + l) * nd + m];
                pixx += cx * (5.0 * cx * cx - 3.0) * t * dw;
                pixy += cy * (5.0 * cx * cx - 1.0) * t * dw;
                piyy += cx * (5.0 * cy * cy - 1.0) * t * dw;
                t = 0.0;
                for (int l = 0; l < nd; ++l) t += vdf[((size_t)d * nt + i) * nd + l] * gy[((size_t)i * nd + l) * nd + m];
                pixx += cy * (5.0 * cx * cx - 1.0) * t * dw;
                pixy += cx * (5.0 * cy * cy - 1.0) * t * dw;
                piyy += cy * (5.0 * cy * cy - 3.0) * t * dw;
            }
            double *o = out + (size_t)i * 7 * nd;
            o[3 * nd + m] = (pixx + 0.5 * piyy) * tc5;
            o[4 * nd + m] = 0.5 * pixy * tc5;
            o[5 * nd + m] = 0.5 * pixy * tc5;
            o[6 * nd + m] = (0.5 * pixx + piyy) * tc5;
        }
}

/* Kinetic wall-trace moments: pybte/acceleration/global_solve.py:31-53.
 * tri_fc_fc[nd][nf][n_tris][3]; out[nk][3*nf]. */
void orc_wall_trace(int ndir, int nt, int nd, int nf, const double *vdf, const double *tri_fc_fc,
                    const double *cxv, const double *cyv, const double *domega, int nk,
                    const int *tri_list, const int *lfc_list, double *out)
{
    for (int k = 0; k < nk; ++k) {
        int tri = tri_list[k], lfc = lfc_list[k];
        for (int m = 0; m < nf; ++m) {
            double tbc = 0.0, qxbc = 0.0, qybc = 0.0;
            for (int d = 0; d < ndir; ++d) {
                double t = 0.0;
                for (int l = 0; l < nd; ++l)
                    t += vdf[((size_t)d * nt + tri) * nd + l] * tri_fc_fc[(((size_t)l * nf + m) * nt + tri) * 3 + lfc];
                tbc += t * domega[d];
                qxbc += cxv[d] * t * domega[d];
                qybc += cyv[d] * t * domega[d];
            }
            out[(size_t)k * 3 * nf + m] = tbc;
            out[(size_t)k * 3 * nf + nf + m] = qxbc;
            out[(size_t)k * 3 * nf + 2 * nf + m] = qybc;
        }
    }
}

/* Damped beta-blend of the HDG solution into the distribution:
 * pybte/acceleration/correction.py:29-75 (defect = 0, the shipped scheme). */
void orc_correct(int ndir, int nt, int nd, double *vdf, const double *uq, const double *cxv,
                 const double *cyv, const double *domega, const double *int_tri, const double *tri_hmin,
                 double cv, double vg, double tau_r, double tau_n, double tau_c, double tau_thr,
                 double pi, int use_hmin, double *ts, double *qxs, double *qys, double *temp,
                 double *qx, double *qy)
{
    double drift = tau_c / tau_n * 3.0 / 4.0 / pi / vg / vg;
    for (int i = 0; i < nt; ++i) {
        double tau_loc = use_hmin ? tau_r / tri_hmin[i] : tau_r;
        double beta = (tau_loc < tau_thr ? tau_loc : tau_thr) / tau_loc;
        temp[i] = 0.0; qx[i] = 0.0; qy[i] = 0.0;
        for (int m = 0; m < nd; ++m) {
            double t_vdf = 0.0, qx_vdf = 0.0, qy_vdf = 0.0;
            for (int d = 0; d < ndir; ++d) {
                double f = vdf[((size_t)d * nt + i) * nd + m];
                t_vdf += f * domega[d];
                qx_vdf += cxv[d] * f * domega[d];
                qy_vdf += cyv[d] * f * domega[d];
            }
            t_vdf = t_vdf / cv;
            double l_t = (uq[(size_t)m * nt + i] - 0.0 - t_vdf) * beta;
            double l_qx = (uq[(size_t)(nd + m) * nt + i] - 0.0 - qx_vdf) * beta;
            double l_qy = (uq[(size_t)(2 * nd + m) * nt + i] - 0.0 - qy_vdf) * beta;
            double eq = l_t * cv / 4.0 / pi;
            for (int d = 0; d < ndir; ++d)
                vdf[((size_t)d * nt + i) * nd + m] = vdf[((size_t)d * nt + i) * nd + m] + eq
                                                     + (cxv[d] * l_qx + cyv[d] * l_qy) * drift;
            ts[(size_t)m * nt + i] = l_t + t_vdf;
            qxs[(size_t)m * nt + i] = l_qx + qx_vdf;
            qys[(size_t)m * nt + i] = l_qy + qy_vdf;
            temp[i] += (l_t + t_vdf) * int_tri[(size_t)m * nt + i];
            qx[i] += (l_qx + qx_vdf) * int_tri[(size_t)m * nt + i];
            qy[i] += (l_qy + qy_vdf) * int_tri[(size_t)m * nt + i];
        }
    }
}
