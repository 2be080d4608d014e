// Context creation: sweep scheduling on the host, operator upload, optional
// precomputed FP64 factors.  Stands in for SweepContext.build / factorise
// (pybte/sweep.py:74-129) and build_sweep_order (pybte/ordering.py:143-175).
//
// Scheduling.  pybte walks each direction's elements in a topological order
// (TRI_ORDER) one at a time.  Without periodic faces or broken cycles, an
// element's solve reads only its upwind neighbours' final values, so every
// topological order gives the same bits; the GPU walks wavefront *levels*
// instead (level = 1 + max level of the upwind neighbours) and solves all
// elements of a level at once.  Directions whose upwind relation agrees on
// every interior face (same sign of c.n) share one level list: they form a
// "class".  On the structured benchmark meshes the face normals take four
// orientations, so all ordinates fall into a handful of classes.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pbte_internal.cuh"

namespace pbte {
std::atomic<long long> g_live_bytes{0};
}

namespace {

template <typename T>
int upload(const T *h, size_t n, T **d, size_t *bytes) {
    if (n == 0) { *d = nullptr; return PBTE_OK; }
    if (cudaMalloc((void **)d, n * sizeof(T)) != cudaSuccess) return PBTE_ERR_NOMEM;
    *bytes += n * sizeof(T);
    pbte::g_live_bytes += (long long)(n * sizeof(T));
    if (cudaMemcpy(*d, h, n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return PBTE_ERR_CUDA;
    return PBTE_OK;
}

template <typename T>
int alloc(size_t n, T **d, size_t *bytes) {
    if (n == 0) { *d = nullptr; return PBTE_OK; }
    if (cudaMalloc((void **)d, n * sizeof(T)) != cudaSuccess) return PBTE_ERR_NOMEM;
    *bytes += n * sizeof(T);
    pbte::g_live_bytes += (long long)(n * sizeof(T));
    return PBTE_OK;
}

int8_t sgn(double v) { return v > 0.0 ? 1 : (v < 0.0 ? -1 : 0); }

// Does face il of element i make it wait for the element behind the face in
// this sweep?  Interior faces with inflow (c.n < 0 on i's side, as pybte's
// ioflag) do; periodic faces do when marked fresh for the class.
inline bool in_sweep_inflow(const pbte_case_desc *d, double cx, double cy, const uint8_t *fresh, int i, int il) {
    const int nb = d->upwind_tri[i * 3 + il];
    const int fc = d->tri_faces[i * 3 + il];
    if (nb < 0) return false;
    if (d->face_bc[fc] >= 0 && !(fresh && ((fresh[i] >> il) & 1))) return false;
    return cx * d->nx[i * 3 + il] + cy * d->ny[i * 3 + il] < 0.0;
}

// Kahn levels of one direction's dependency graph (level = 1 + the deepest
// element it waits for).  Returns false on a cycle.
bool levels_for(const pbte_case_desc *d, double cx, double cy, const uint8_t *fresh,
                std::vector<int32_t> &level, std::vector<int32_t> &indeg, std::vector<int32_t> &queue,
                std::vector<int32_t> &succ_ptr, std::vector<int32_t> &succ) {
    const int nt = d->n_tris;
    level.assign(nt, 0);
    indeg.assign(nt, 0);
    succ_ptr.assign(nt + 1, 0);
    for (int i = 0; i < nt; ++i)
        for (int il = 0; il < 3; ++il)
            if (in_sweep_inflow(d, cx, cy, fresh, i, il)) {
                indeg[i]++;
                succ_ptr[d->upwind_tri[i * 3 + il] + 1]++;
            }
    for (int i = 0; i < nt; ++i) succ_ptr[i + 1] += succ_ptr[i];
    succ.assign(succ_ptr[nt], 0);
    std::vector<int32_t> fill(succ_ptr.begin(), succ_ptr.end() - 1);
    for (int i = 0; i < nt; ++i)
        for (int il = 0; il < 3; ++il)
            if (in_sweep_inflow(d, cx, cy, fresh, i, il)) succ[fill[d->upwind_tri[i * 3 + il]]++] = i;
    queue.clear();
    for (int i = 0; i < nt; ++i)
        if (indeg[i] == 0) queue.push_back(i);
    size_t head = 0;
    while (head < queue.size()) {
        const int i = queue[head++];
        for (int e = succ_ptr[i]; e < succ_ptr[i + 1]; ++e) {
            const int j = succ[e];
            level[j] = std::max(level[j], level[i] + 1);
            if (--indeg[j] == 0) queue.push_back(j);
        }
    }
    return (int)queue.size() == nt;
}

// pybte's TRI_ORDER position of every element for one direction
// (pybte/ordering.py:61-140, without cycle breaking): rescan the elements in
// ascending index, emit each one with no incoming interior face left, and
// clear the matching flag of its neighbours at once, so a later element of
// the same scan can follow it.  Returns false on a cycle.
bool reference_order(const pbte_case_desc *d, double cx, double cy, std::vector<int32_t> &pos) {
    const int nt = d->n_tris;
    std::vector<int8_t> io((size_t)nt * 3, 0);
    for (int i = 0; i < nt; ++i)
        for (int il = 0; il < 3; ++il) {
            const int fc = d->tri_faces[i * 3 + il];
            if (d->upwind_tri[i * 3 + il] < 0 || d->face_bc[fc] >= 0) continue;
            const double flux = cx * d->nx[i * 3 + il] + cy * d->ny[i * 3 + il];
            io[i * 3 + il] = flux > 0.0 ? 1 : (flux < 0.0 ? -1 : 0);
        }
    std::vector<char> queued(nt, 1);
    pos.assign(nt, -1);
    int num = 0;
    while (num < nt) {
        bool progressed = false;
        for (int i = 0; i < nt; ++i) {
            if (!queued[i] || io[i * 3] == -1 || io[i * 3 + 1] == -1 || io[i * 3 + 2] == -1) continue;
            pos[i] = num++;
            queued[i] = 0;
            progressed = true;
            for (int il = 0; il < 3; ++il) {
                const int fc = d->tri_faces[i * 3 + il];
                const int t2 = d->upwind_tri[i * 3 + il];
                if (t2 < 0 || d->face_bc[fc] >= 0) continue;
                for (int k = 0; k < 3; ++k)
                    if (d->face_bc[d->tri_faces[t2 * 3 + k]] < 0 && d->upwind_tri[t2 * 3 + k] == i) {
                        io[t2 * 3 + k] = 0;
                        break;
                    }
            }
        }
        if (!progressed) return false;
    }
    return true;
}

// Direction classes: the sign pattern of c.n over the interior and periodic
// faces (each face seen from its first side), hashed (FNV-1a) and then
// compared in full against the class representative; classes are numbered
// by first appearance.  A face's sign depends only on the exact bits of its
// normal, so the pattern is taken over the distinct normals (a handful on
// structured meshes, at most one per face): the same classes as face by face.
void direction_classes(const pbte_case_desc *d, std::vector<int32_t> &dir_class, std::vector<int> &class_rep) {
    std::vector<double> unx, uny;
    {
        std::unordered_map<uint64_t, std::vector<int>> seen;   // hash of the bits -> distinct ids
        auto bits = [](double v) { uint64_t u; std::memcpy(&u, &v, sizeof u); return u; };
        for (int f = 0; f < d->n_faces; ++f) {
            const int bc = d->face_bc[f];
            if (!(bc < 0 || d->bc_type[bc] == 3)) continue;
            const int t = d->face_tri[f * 2 + 0] >= 0 ? d->face_tri[f * 2 + 0] : d->face_tri[f * 2 + 1];
            const int l = d->face_tri[f * 2 + 0] >= 0 ? d->face_lfc[f * 2 + 0] : d->face_lfc[f * 2 + 1];
            const double nx = d->nx[t * 3 + l], ny = d->ny[t * 3 + l];
            const uint64_t h = bits(nx) * 0x9E3779B97F4A7C15ull ^ bits(ny);
            auto &ids = seen[h];
            bool dup = false;
            for (int q : ids)
                if (bits(unx[q]) == bits(nx) && bits(uny[q]) == bits(ny)) { dup = true; break; }
            if (dup) continue;
            ids.push_back((int)unx.size());
            unx.push_back(nx);
            uny.push_back(ny);
        }
    }
    auto pattern = [&](int dir, std::vector<int8_t> &p) {
        p.resize(unx.size());
        for (size_t k = 0; k < unx.size(); ++k) p[k] = sgn(d->cxv[dir] * unx[k] + d->cyv[dir] * uny[k]);
    };
    std::unordered_multimap<uint64_t, int> by_hash;  // hash -> class id
    class_rep.clear();
    dir_class.assign(d->ndir, 0);
    std::vector<int8_t> pat, pat2;
    for (int dir = 0; dir < d->ndir; ++dir) {
        pattern(dir, pat);
        uint64_t h = 1469598103934665603ull;
        for (int8_t v : pat) { h ^= (uint8_t)v; h *= 1099511628211ull; }
        int found = -1;
        auto range = by_hash.equal_range(h);
        for (auto it = range.first; it != range.second && found < 0; ++it) {
            pattern(class_rep[it->second], pat2);
            if (pat2 == pat) found = it->second;
        }
        if (found < 0) {
            found = (int)class_rep.size();
            class_rep.push_back(dir);
            by_hash.emplace(h, found);
        }
        dir_class[dir] = found;
    }
}

// face arrays a case description must hold for the host-side scheduling
bool desc_faces_valid(const pbte_case_desc *d) {
    if (!d->face_bc || !d->face_tri || !d->face_lfc || !d->nx || !d->ny || !d->cxv || !d->cyv ||
        (d->nbc > 0 && !d->bc_type))
        return false;
    for (int f = 0; f < d->n_faces; ++f) {
        const int bc = d->face_bc[f];
        if (bc >= d->nbc) return false;
        for (int side = 0; side < 2; ++side) {
            const int t = d->face_tri[f * 2 + side], l = d->face_lfc[f * 2 + side];
            if (t >= d->n_tris || (t >= 0 && (l < 0 || l > 2))) return false;
        }
        if (d->face_tri[f * 2] < 0 && d->face_tri[f * 2 + 1] < 0) return false;
    }
    return true;
}

}  // namespace

static int direction_classes_impl(const pbte_case_desc *d, int32_t *dir_class, int32_t *n_classes) {
    if (!d || !dir_class || !n_classes || d->n_tris <= 0 || d->ndir <= 0 || d->n_faces <= 0) return PBTE_ERR_ARG;
    if (!desc_faces_valid(d)) return PBTE_ERR_ARG;
    std::vector<int32_t> cls;
    std::vector<int> rep;
    direction_classes(d, cls, rep);
    std::memcpy(dir_class, cls.data(), sizeof(int32_t) * cls.size());
    *n_classes = (int32_t)rep.size();
    return PBTE_OK;
}

static int direction_levels_impl(const pbte_case_desc *d, int32_t dir, int32_t *level, int32_t *n_levels) {
    if (!d || !level || !n_levels || d->n_tris <= 0 || d->n_faces <= 0 || dir < 0 || dir >= d->ndir)
        return PBTE_ERR_ARG;
    if (!desc_faces_valid(d) || !d->tri_faces || !d->upwind_tri) return PBTE_ERR_ARG;
    const int nt = d->n_tris;
    for (int i = 0; i < nt * 3; ++i) {
        const int fc = d->tri_faces[i], nb = d->upwind_tri[i];
        if (fc < 0 || fc >= d->n_faces || nb >= nt) return PBTE_ERR_ARG;
    }
    const double cx = d->cxv[dir], cy = d->cyv[dir];
    std::vector<uint8_t> fresh;
    bool periodic = false;
    for (int f = 0; f < d->n_faces && !periodic; ++f) periodic = d->face_bc[f] >= 0 && d->bc_type[d->face_bc[f]] == 3;
    if (periodic) {
        // the rule pbte_ctx_create applies per direction class
        std::vector<int32_t> rpos;
        if (!reference_order(d, cx, cy, rpos)) return PBTE_ERR_CYCLE;
        fresh.assign(nt, 0);
        for (int i = 0; i < nt; ++i)
            for (int il = 0; il < 3; ++il) {
                const int fc = d->tri_faces[i * 3 + il];
                const int bc = d->face_bc[fc];
                if (bc < 0 || d->bc_type[bc] != 3) continue;
                const int p = d->upwind_tri[i * 3 + il];
                if (p < 0) continue;
                const double s = cx * d->nx[i * 3 + il] + cy * d->ny[i * 3 + il];
                if (s < 0.0 && rpos[p] < rpos[i]) fresh[i] |= (uint8_t)(1u << il);
            }
    }
    std::vector<int32_t> lv, indeg, queue, succ_ptr, succ;
    if (!levels_for(d, cx, cy, periodic ? fresh.data() : nullptr, lv, indeg, queue, succ_ptr, succ))
        return PBTE_ERR_CYCLE;
    int nlev = 0;
    for (int i = 0; i < nt; ++i) {
        level[i] = lv[i];
        nlev = std::max(nlev, lv[i] + 1);
    }
    *n_levels = nlev;
    return PBTE_OK;
}

extern "C" int pbte_direction_classes(const pbte_case_desc *d, int32_t *dir_class, int32_t *n_classes) {
    try {
        return direction_classes_impl(d, dir_class, n_classes);
    } catch (...) {
        return PBTE_ERR_NOMEM;
    }
}

extern "C" int pbte_direction_levels(const pbte_case_desc *d, int32_t dir, int32_t *level, int32_t *n_levels) {
    try {
        return direction_levels_impl(d, dir, level, n_levels);
    } catch (...) {
        return PBTE_ERR_NOMEM;
    }
}

extern "C" int pbte_ctx_destroy(pbte_ctx *c) {
    if (!c) return PBTE_OK;
    void *ptrs[] = {c->d_cx, c->d_cy, c->d_w, c->d_cells64, c->d_cells32, c->d_ref64, c->d_ref32,
                    c->d_edofs, c->d_dir_class, c->d_class_lvl_off, c->d_class_nlev, c->d_lvl_ptr,
                    c->d_lvl_cells, c->d_int_tri, c->d_wall_ad, c->d_S64, c->d_S32, c->d_lu,
                    c->d_piv, c->d_red, c->d_singular, c->d_up_slot, c->d_class_W, c->d_class_R,
                    c->d_udir_rep, c->d_udir_twin, c->d_rf64, c->d_rf32, c->d_ri, c->d_mom_part,
                    c->d_cx32, c->d_cy32, c->d_w32, c->d_udir_of, c->d_uw32, c->d_ucx32, c->d_ucy32,
                    c->d_uw64, c->d_ucx64, c->d_ucy64, c->d_fresh, c->d_pface, c->d_ptri, c->d_pslot,
                    c->d_psnap, c->d_gsis, c->d_lu32, c->d_tickets};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    pbte::g_live_bytes -= (long long)c->device_bytes;
    delete c;
    return PBTE_OK;
}

namespace {
// Owns a context under construction: destroys it unless released.
struct CtxGuard {
    pbte_ctx *c;
    ~CtxGuard() {
        if (c) pbte_ctx_destroy(c);
    }
    pbte_ctx *release() {
        pbte_ctx *p = c;
        c = nullptr;
        return p;
    }
};
}  // namespace

static int ctx_create_impl(const pbte_case_desc *d, int precompute, pbte_ctx **out) {
    if (!d || !out) return PBTE_ERR_ARG;
    *out = nullptr;
    const int nt = d->n_tris, nd = d->ndof, nf = d->ndof_fc, ndir = d->ndir;
    int deg = nf - 1;
    if (nt <= 0 || ndir <= 0 || d->n_faces <= 0 || deg < 1 || deg > 4 ||
        nd != (deg + 1) * (deg + 2) / 2)
        return PBTE_ERR_ARG;
    // the guard destroys the half-built context on every early return and on
    // a C++ exception (a failed host allocation), so neither leaks it
    CtxGuard guard{new pbte_ctx()};
    pbte_ctx *c = guard.c;
    if (cudaGetDevice(&c->device) != cudaSuccess) return PBTE_ERR_CUDA;
    c->n_tris = nt; c->n_faces = d->n_faces; c->nd = nd; c->nf = nf; c->ndir = ndir;
    c->nbc = d->nbc; c->deg = deg;
    c->cv = d->cv; c->vg = d->vg; c->tau_r = d->tau_r; c->tau_n = d->tau_n; c->tau_c = d->tau_c;
    c->h_cx.assign(d->cxv, d->cxv + ndir);
    c->h_cy.assign(d->cyv, d->cyv + ndir);
    c->h_w.assign(d->domega, d->domega + ndir);
    int rc = PBTE_OK;
#define TRY(x) do { rc = (x); if (rc != PBTE_OK) return rc; } while (0)

    // ---- element records -------------------------------------------------
    std::vector<pbte::CellRec<double>> r64(nt);
    std::vector<pbte::CellRec<float>> r32(nt);
    const double four_pi = 4.0 * pbte::kPi;
    for (int i = 0; i < nt; ++i) {
        auto &r = r64[i];
        std::memset(&r, 0, sizeof(r));
        r.area2 = d->area2[i];
        r.gxa = d->dxi[i * 2 + 0]; r.gxb = d->dxi[i * 2 + 1];
        r.gya = d->deta[i * 2 + 0]; r.gyb = d->deta[i * 2 + 1];
        for (int il = 0; il < 3; ++il) {
            r.es[il] = d->edge_scale[i * 3 + il];
            r.nx[il] = d->nx[i * 3 + il];
            r.ny[il] = d->ny[i * 3 + il];
            int fc = d->tri_faces[i * 3 + il];
            if (fc < 0 || fc >= d->n_faces) { return PBTE_ERR_ARG; }
            r.face[il] = fc;
            r.upw[il] = d->upwind_tri[i * 3 + il];
            int bc = d->face_bc[fc];
            if (bc < 0) {
                r.kind[il] = 0;
                if (r.upw[il] < 0 || r.upw[il] >= nt) { return PBTE_ERR_ARG; }
            } else {
                if (bc >= d->nbc) { return PBTE_ERR_ARG; }
                int t = d->bc_type[bc];
                if (t == 1) { r.kind[il] = 1; r.bval[il] = d->cv / four_pi * d->bc_temp[bc]; }
                else if (t == 2) r.kind[il] = 2;
                else if (t == 3) { r.kind[il] = 3; c->has_periodic = true; }
                else { return PBTE_ERR_UNSUPPORTED; }
            }
            for (int b = 0; b < nf; ++b) {
                int v = r.upw[il] >= 0 ? d->edge_map[(i * 3 + il) * nf + b] : 0;
                if (v < 0 || v >= nd) v = 0;
                r.emap[il][b] = (int8_t)v;
            }
        }
        auto &q = r32[i];
        std::memset(&q, 0, sizeof(q));
        q.area2 = (float)r.area2; q.gxa = (float)r.gxa; q.gxb = (float)r.gxb;
        q.gya = (float)r.gya; q.gyb = (float)r.gyb;
        for (int il = 0; il < 3; ++il) {
            q.es[il] = (float)r.es[il]; q.nx[il] = (float)r.nx[il]; q.ny[il] = (float)r.ny[il];
            q.bval[il] = (float)r.bval[il]; q.face[il] = r.face[il]; q.upw[il] = r.upw[il];
            q.kind[il] = r.kind[il];
            for (int b = 0; b < pbte::kMaxNf; ++b) q.emap[il][b] = r.emap[il][b];
        }
    }
    TRY(upload(r64.data(), (size_t)nt, &c->d_cells64, &c->device_bytes));
    TRY(upload(r32.data(), (size_t)nt, &c->d_cells32, &c->device_bytes));

    // ---- reference matrices, edge DOFs, ordinates -----------------------
    std::vector<double> ref(6 * nd * nd);
    std::memcpy(ref.data(), d->ref_mass, sizeof(double) * nd * nd);
    std::memcpy(ref.data() + nd * nd, d->ref_dx, sizeof(double) * nd * nd);
    std::memcpy(ref.data() + 2 * nd * nd, d->ref_dy, sizeof(double) * nd * nd);
    std::memcpy(ref.data() + 3 * nd * nd, d->ref_edge, sizeof(double) * 3 * nd * nd);
    std::vector<float> ref32(ref.begin(), ref.end());
    TRY(upload(ref.data(), ref.size(), &c->d_ref64, &c->device_bytes));
    TRY(upload(ref32.data(), ref32.size(), &c->d_ref32, &c->device_bytes));
    TRY(upload(d->edge_dofs, (size_t)3 * nf, &c->d_edofs, &c->device_bytes));
    TRY(upload(d->cxv, (size_t)ndir, &c->d_cx, &c->device_bytes));
    TRY(upload(d->cyv, (size_t)ndir, &c->d_cy, &c->device_bytes));
    TRY(upload(d->domega, (size_t)ndir, &c->d_w, &c->device_bytes));
    {
        std::vector<float> a(d->cxv, d->cxv + ndir), b(d->cyv, d->cyv + ndir), w(d->domega, d->domega + ndir);
        TRY(upload(a.data(), a.size(), &c->d_cx32, &c->device_bytes));
        TRY(upload(b.data(), b.size(), &c->d_cy32, &c->device_bytes));
        TRY(upload(w.data(), w.size(), &c->d_w32, &c->device_bytes));
    }
    TRY(upload(d->int_tri, (size_t)nd * nt, &c->d_int_tri, &c->device_bytes));

    // ---- adiabatic wall faces -------------------------------------------
    std::vector<pbte::WallFace> walls;
    for (int f = 0; f < d->n_faces; ++f) {
        int bc = d->face_bc[f];
        if (bc < 0 || d->bc_type[bc] != 2) continue;
        pbte::WallFace w{};
        w.face = f;
        if (d->face_tri[f * 2 + 0] < 0) { w.tri = d->face_tri[f * 2 + 1]; w.lfc = d->face_lfc[f * 2 + 1]; }
        else { w.tri = d->face_tri[f * 2 + 0]; w.lfc = d->face_lfc[f * 2 + 0]; }
        w.nx = -d->nx[w.tri * 3 + w.lfc];
        w.ny = -d->ny[w.tri * 3 + w.lfc];
        walls.push_back(w);
    }
    c->n_wall_ad = (int)walls.size();
    TRY(upload(walls.data(), walls.size(), &c->d_wall_ad, &c->device_bytes));

    // ---- periodic faces ---------------------------------------------------
    std::vector<int32_t> pface, ptri, pslot(d->n_faces, -1);
    for (int f = 0; f < d->n_faces; ++f) {
        const int bc = d->face_bc[f];
        if (bc < 0 || d->bc_type[bc] != 3) continue;
        const int side = d->face_tri[f * 2 + 0] >= 0 ? 0 : 1;
        const int t = d->face_tri[f * 2 + side], l = d->face_lfc[f * 2 + side];
        const int partner = d->upwind_tri[t * 3 + l];
        if (partner < 0 || partner >= nt) { return PBTE_ERR_ARG; }
        pslot[f] = (int32_t)pface.size();
        pface.push_back(f);
        ptri.push_back(partner);
    }
    c->n_pfaces = (int)pface.size();
    if (c->n_pfaces) {
        TRY(upload(pface.data(), pface.size(), &c->d_pface, &c->device_bytes));
        TRY(upload(ptri.data(), ptri.size(), &c->d_ptri, &c->device_bytes));
        TRY(upload(pslot.data(), pslot.size(), &c->d_pslot, &c->device_bytes));
        TRY(alloc((size_t)ndir * c->n_pfaces * nd, &c->d_psnap, &c->device_bytes));
    }

    // ---- direction classes and wavefront levels -------------------------
    std::vector<int> class_rep;
    std::vector<int32_t> dir_class;
    direction_classes(d, dir_class, class_rep);
    c->nclass = (int)class_rep.size();
    std::vector<int32_t> lvl_cells((size_t)c->nclass * nt), lvl_ptr, class_off(c->nclass),
        class_nlev(c->nclass);
    const size_t M = (size_t)c->nclass * nt;   // field stride of the sweep records
    std::vector<double> rf64(M * pbte::kNumRecReal);
    std::vector<float> rf32(M * pbte::kNumRecReal);
    std::vector<int32_t> ri(M * pbte::kNumRecInt);
    constexpr int kNearDepth = 4;
    // ring of upwind values in shared memory: slot (level % R) * W + position,
    // R = 1 + the largest level gap of an in-sweep dependency, W = widest level
    std::vector<int32_t> up_slot((size_t)c->nclass * nt * 3, -1), class_W(c->nclass), class_R(c->nclass);
    std::vector<uint8_t> fresh(c->n_pfaces ? (size_t)c->nclass * nt : 0, 0);
    // The classes are independent: each builds its levels, ring slots and
    // records into its own stretch of the shared arrays, on host threads.
    struct ClassOut {
        int status = PBTE_OK, nlev = 0, W = 0, R = 1, nfar = 0;
        std::vector<int32_t> count;   // level offsets within the class, nlev + 1
    };
    std::vector<ClassOut> cls_out(c->nclass);
    auto build_class = [&](int k, ClassOut &o) {
        std::vector<int32_t> level, indeg, queue, count, pos(nt), far_idx, succ_ptr, succ, rpos;
        int dir = class_rep[k];
        uint8_t *fr = c->n_pfaces ? fresh.data() + (size_t)k * nt : nullptr;
        if (fr) {
            // a periodic inflow reads this sweep's partner value when the
            // partner comes first in pybte's order for these directions
            if (!reference_order(d, d->cxv[dir], d->cyv[dir], rpos)) { o.status = PBTE_ERR_CYCLE; return; }
            for (int i = 0; i < nt; ++i)
                for (int il = 0; il < 3; ++il) {
                    const int fc = d->tri_faces[i * 3 + il];
                    if (pslot[fc] < 0) continue;
                    const int p = d->upwind_tri[i * 3 + il];
                    const double s = d->cxv[dir] * d->nx[i * 3 + il] + d->cyv[dir] * d->ny[i * 3 + il];
                    if (s < 0.0 && rpos[p] < rpos[i]) fr[i] |= (uint8_t)(1u << il);
                }
        }
        if (!levels_for(d, d->cxv[dir], d->cyv[dir], fr, level, indeg, queue, succ_ptr, succ)) {
            o.status = PBTE_ERR_CYCLE;
            return;
        }
        int nlev = 0;
        for (int i = 0; i < nt; ++i) nlev = std::max(nlev, level[i] + 1);
        count.assign(nlev + 1, 0);
        for (int i = 0; i < nt; ++i) count[level[i] + 1]++;
        int W = 0;
        for (int L = 0; L < nlev; ++L) W = std::max(W, count[L + 1]);
        for (int L = 0; L < nlev; ++L) count[L + 1] += count[L];
        std::vector<int32_t> fill(count.begin(), count.end() - 1);
        for (int i = 0; i < nt; ++i) {
            pos[i] = fill[level[i]] - count[level[i]];
            lvl_cells[(size_t)k * nt + fill[level[i]]++] = i;
        }
        // near ring of at most kNearDepth levels; an upwind value needed further
        // ahead (rare: near the lines where the mesh diagonals flip) is also
        // kept in a dedicated far slot
        int R = 1;
        const double cx = d->cxv[dir], cy = d->cyv[dir];
        for (int i = 0; i < nt; ++i)
            for (int il = 0; il < 3; ++il)
                if (in_sweep_inflow(d, cx, cy, fr, i, il))
                    R = std::max(R, level[i] - level[d->upwind_tri[i * 3 + il]] + 1);
        R = std::min(R, kNearDepth);
        class_W[k] = W;
        class_R[k] = R;
        far_idx.assign(nt, -1);
        int nfar = 0;
        for (int i = 0; i < nt; ++i) {
            size_t p = (size_t)k * nt + count[level[i]] + pos[i];
            for (int il = 0; il < 3; ++il) {
                if (!in_sweep_inflow(d, cx, cy, fr, i, il)) continue;
                const int nb = d->upwind_tri[i * 3 + il];
                if (level[i] - level[nb] < R) {
                    up_slot[p * 3 + il] = (level[nb] % R) * W + pos[nb];
                } else {
                    if (far_idx[nb] < 0) far_idx[nb] = nfar++;
                    up_slot[p * 3 + il] = -2 - far_idx[nb];
                }
            }
        }
        for (int p = 0; p < nt; ++p) {
            const size_t kp = (size_t)k * nt + p;
            const int i = lvl_cells[kp];
            const auto &a = r64[i];
            const auto &b32 = r32[i];
            auto put = [&](int f, double v64, float v32) {
                rf64[f * M + kp] = v64;
                rf32[f * M + kp] = v32;
            };
            put(pbte::kRA2, a.area2, b32.area2);
            put(pbte::kRGxa, a.gxa, b32.gxa);
            put(pbte::kRGxb, a.gxb, b32.gxb);
            put(pbte::kRGya, a.gya, b32.gya);
            put(pbte::kRGyb, a.gyb, b32.gyb);
            uint32_t kinds = 0;
            for (int il = 0; il < 3; ++il) {
                put(pbte::kREs + il, a.es[il], b32.es[il]);
                put(pbte::kRNx + il, a.nx[il], b32.nx[il]);
                put(pbte::kRNy + il, a.ny[il], b32.ny[il]);
                put(pbte::kRBval + il, a.bval[il], b32.bval[il]);
                ri[(pbte::kIUp + il) * M + kp] = up_slot[kp * 3 + il];
                uint32_t packed = 0;
                for (int b = 0; b < nf; ++b) packed |= (uint32_t)(a.emap[il][b] & 15) << (4 * b);
                ri[(pbte::kIEmp + il) * M + kp] = (int32_t)packed;
                ri[(pbte::kIFace + il) * M + kp] = a.face[il];
                const int kind = (a.kind[il] == 3 && fr && ((fr[i] >> il) & 1)) ? 4 : a.kind[il];
                kinds |= (uint32_t)(uint8_t)kind << (8 * il);
            }
            ri[pbte::kICell * M + kp] = i;
            ri[pbte::kIFarOut * M + kp] = far_idx[i];
            ri[pbte::kIKind * M + kp] = (int32_t)kinds;
        }
        o.nlev = nlev;
        o.W = W;
        o.R = R;
        o.nfar = nfar;
        o.count = std::move(count);
    };
    {
        std::atomic<int> next{0};
        auto worker = [&]() {
            for (int k = next++; k < c->nclass; k = next++) {
                try {
                    build_class(k, cls_out[k]);
                } catch (...) {
                    // host allocation failed: reported as a status, no
                    // exception leaves the worker (or the C ABI)
                    cls_out[k].status = PBTE_ERR_NOMEM;
                }
            }
        };
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const int nth = (int)std::min<unsigned>({hw, 16u, (unsigned)c->nclass});
        std::vector<std::thread> pool;
        try {
            for (int t = 1; t < nth; ++t) pool.emplace_back(worker);
        } catch (...) {
            // no more threads: the calling thread takes the remaining classes
        }
        worker();
        for (auto &th : pool) th.join();
    }
    for (int k = 0; k < c->nclass; ++k) {
        const ClassOut &o = cls_out[k];
        if (o.status != PBTE_OK) { return o.status; }
        class_off[k] = (int32_t)lvl_ptr.size();
        class_nlev[k] = o.nlev;
        for (int L = 0; L <= o.nlev; ++L) lvl_ptr.push_back(o.count[L] + k * nt);
        c->far_max = std::max(c->far_max, o.nfar);
        c->nlev_max = std::max(c->nlev_max, o.nlev);
        c->ring_W = std::max(c->ring_W, o.W);
        c->ring_R = std::max(c->ring_R, o.R);
    }
    // z-mirror twins: ordinates with the same in-plane velocity (and weight)
    // see the same transport; one block sweeps the pair and stores both
    std::vector<int32_t> urep, utwin;
    std::vector<char> used(ndir, 0);
    for (int a = 0; a < ndir; ++a) {
        if (used[a]) continue;
        used[a] = 1;
        int tw = -1;
        for (int b = a + 1; b < ndir && tw < 0; ++b)
            if (!used[b] && dir_class[b] == dir_class[a] && std::fabs(d->cxv[a] - d->cxv[b]) <= 1e-12 &&
                std::fabs(d->cyv[a] - d->cyv[b]) <= 1e-12)
                tw = b;
        if (tw >= 0) used[tw] = 1;
        urep.push_back(a);
        utwin.push_back(tw);
    }
    c->n_udir = (int)urep.size();
    std::vector<int32_t> udir_of(ndir, 0);
    for (int u = 0; u < c->n_udir; ++u) {
        udir_of[urep[u]] = u;
        if (utwin[u] >= 0) udir_of[utwin[u]] = u;
    }
    TRY(upload(udir_of.data(), udir_of.size(), &c->d_udir_of, &c->device_bytes));
    {
        // folded weights: a twin pair contributes w_a f + w_b f = (w_a + w_b) f
        std::vector<double> uw(c->n_udir), ucx(c->n_udir), ucy(c->n_udir);
        for (int u = 0; u < c->n_udir; ++u) {
            uw[u] = d->domega[urep[u]] + (utwin[u] >= 0 ? d->domega[utwin[u]] : 0.0);
            ucx[u] = d->cxv[urep[u]];
            ucy[u] = d->cyv[urep[u]];
        }
        std::vector<float> uw32(uw.begin(), uw.end()), ucx32(ucx.begin(), ucx.end()), ucy32(ucy.begin(), ucy.end());
        TRY(upload(uw.data(), uw.size(), &c->d_uw64, &c->device_bytes));
        TRY(upload(ucx.data(), ucx.size(), &c->d_ucx64, &c->device_bytes));
        TRY(upload(ucy.data(), ucy.size(), &c->d_ucy64, &c->device_bytes));
        TRY(upload(uw32.data(), uw32.size(), &c->d_uw32, &c->device_bytes));
        TRY(upload(ucx32.data(), ucx32.size(), &c->d_ucx32, &c->device_bytes));
        TRY(upload(ucy32.data(), ucy32.size(), &c->d_ucy32, &c->device_bytes));
    }
    TRY(upload(dir_class.data(), dir_class.size(), &c->d_dir_class, &c->device_bytes));
    TRY(upload(class_off.data(), class_off.size(), &c->d_class_lvl_off, &c->device_bytes));
    TRY(upload(class_nlev.data(), class_nlev.size(), &c->d_class_nlev, &c->device_bytes));
    TRY(upload(lvl_ptr.data(), lvl_ptr.size(), &c->d_lvl_ptr, &c->device_bytes));
    TRY(upload(lvl_cells.data(), lvl_cells.size(), &c->d_lvl_cells, &c->device_bytes));
    TRY(upload(up_slot.data(), up_slot.size(), &c->d_up_slot, &c->device_bytes));
    TRY(upload(rf64.data(), rf64.size(), &c->d_rf64, &c->device_bytes));
    TRY(upload(rf32.data(), rf32.size(), &c->d_rf32, &c->device_bytes));
    TRY(upload(ri.data(), ri.size(), &c->d_ri, &c->device_bytes));
    TRY(upload(class_W.data(), class_W.size(), &c->d_class_W, &c->device_bytes));
    TRY(upload(class_R.data(), class_R.size(), &c->d_class_R, &c->device_bytes));
    TRY(upload(urep.data(), urep.size(), &c->d_udir_rep, &c->device_bytes));
    TRY(upload(utwin.data(), utwin.size(), &c->d_udir_twin, &c->device_bytes));
    if (!fresh.empty()) TRY(upload(fresh.data(), fresh.size(), &c->d_fresh, &c->device_bytes));

    // ---- scratch ----------------------------------------------------------
    TRY(alloc((size_t)3 * nd * nt, &c->d_S64, &c->device_bytes));
    TRY(alloc((size_t)3 * nd * nt, &c->d_S32, &c->device_bytes));
    TRY(alloc((size_t)4096, &c->d_red, &c->device_bytes));
    TRY(alloc((size_t)((ndir + 31) / 32) * 3 * nd * nt, &c->d_mom_part, &c->device_bytes));
    TRY(alloc((size_t)4 * nd * nt, &c->d_gsis, &c->device_bytes));
    TRY(alloc((size_t)(nt + 31) / 32, &c->d_tickets, &c->device_bytes));
    if (cudaMemset(c->d_tickets, 0, sizeof(uint32_t) * ((nt + 31) / 32)) != cudaSuccess) {
        return PBTE_ERR_CUDA;
    }
    TRY(alloc((size_t)1, &c->d_singular, &c->device_bytes));
    if (cudaMemset(c->d_singular, 0, sizeof(int32_t)) != cudaSuccess) { return PBTE_ERR_CUDA; }

    if (precompute) {
        TRY(alloc(pbte::factor_count(c->n_udir, nt, nd * nd), &c->d_lu, &c->device_bytes));
        TRY(alloc(pbte::factor_count(c->n_udir, nt, nd), &c->d_piv, &c->device_bytes));
        TRY(pbte::launch_factorise(c, 0));
        int32_t bad = 0;
        if (cudaMemcpy(&bad, c->d_singular, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) {
            return PBTE_ERR_CUDA;
        }
        if (bad) { return PBTE_ERR_SINGULAR; }
    }
    if (cudaDeviceSynchronize() != cudaSuccess) { return PBTE_ERR_CUDA; }
#undef TRY
    *out = guard.release();
    return PBTE_OK;
}

// No C++ exception leaves the C ABI: a failed host allocation is a status.
extern "C" int pbte_ctx_create(const pbte_case_desc *d, int precompute, pbte_ctx **out) {
    try {
        return ctx_create_impl(d, precompute, out);
    } catch (...) {
        if (out) *out = nullptr;
        return PBTE_ERR_NOMEM;
    }
}

extern "C" int pbte_singular_count(pbte_ctx *c, int64_t *count, int reset) {
    if (!c || !count) return PBTE_ERR_ARG;
    int32_t v = 0;
    if (cudaMemcpy(&v, c->d_singular, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) return PBTE_ERR_CUDA;
    *count = v;
    if (reset && cudaMemset(c->d_singular, 0, sizeof(int32_t)) != cudaSuccess) return PBTE_ERR_CUDA;
    return PBTE_OK;
}

extern "C" int pbte_device_bytes_live(int64_t *bytes) {
    if (!bytes) return PBTE_ERR_ARG;
    *bytes = pbte::g_live_bytes.load();
    return PBTE_OK;
}

extern "C" int pbte_ctx_info(const pbte_ctx *c, int64_t *nlev, int64_t *ncls, int64_t *bytes) {
    if (!c) return PBTE_ERR_ARG;
    if (nlev) *nlev = c->nlev_max;
    if (ncls) *ncls = c->nclass;
    if (bytes) *bytes = (int64_t)c->device_bytes;
    return PBTE_OK;
}
