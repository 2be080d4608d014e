"""Host side of the nested-dissection trace solve: the dissection tree, the
multifrontal factors and the layout the device kernels read, checked by
restating the two device sweeps in numpy (the kernels' arithmetic, row by
row) on block-sparse matrices with the GSIS trace pattern (a dense block
for every two faces of one element, plus the periodic pairs), against
scipy's sparse LU."""
import numpy as np
import pytest
import scipy.sparse as sp
from scipy.sparse.linalg import spsolve

from cases import periodic_case, small_case
from pbte_gb300.discretisation import Discretisation
from pbte_gb300.trace_nd import NestedDissectionSolver, dissect


def trace_pattern_matrix(mesh, b, seed, periodic=False):
    rng = np.random.default_rng(seed)
    nf = mesh.n_faces
    rows, cols, vals = [], [], []
    rr, cc = np.meshgrid(np.arange(b), np.arange(b), indexing="ij")
    for t in range(mesh.n_tris):
        for fi in mesh.tri_faces[t]:
            for fj in mesh.tri_faces[t]:
                rows.append(fi * b + rr.ravel())
                cols.append(fj * b + cc.ravel())
                vals.append(rng.standard_normal(b * b))
    if periodic:
        pair = np.asarray(mesh.face_pair)
        for f in np.flatnonzero(pair >= 0):
            rows.append(f * b + rr.ravel())
            cols.append(pair[f] * b + cc.ravel())
            vals.append(rng.standard_normal(b * b))
    K = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(nf * b, nf * b))
    K = K.tocsr()
    K.sum_duplicates()
    K = K + sp.diags(np.asarray(abs(K).sum(axis=1)).ravel() + 1.0)
    return K.tocsr()


def emulate_solve(s: NestedDissectionSolver, rhs: np.ndarray) -> np.ndarray:
    """pbte_nd_forward / pbte_nd_backward restated with the solver's arrays."""
    meta, idx = s.meta.numpy(), s.idx.numpy()
    cptr, csrc = s.cptr.numpy(), s.csrc.numpy()
    G, H = s.Gd.numpy(), s.Hd.numpy()
    z = np.zeros(s.n)
    x = np.zeros(s.n)
    delta = np.zeros(s.delta.numel())

    def upd(at):
        return delta[csrc[cptr[at]:cptr[at + 1]]].sum()

    for items, n_items, *_ in s.levels:
        for node, r0, r1, _ in items.numpy()[:n_items]:
            ioff, o, m, goff, _, doff, coff, _ = meta[node]
            Gt = G[goff:goff + o * m].reshape(o, m)          # G stored column-major
            v = np.array([rhs[idx[ioff + p]] + upd(coff + p) for p in range(o)])
            for r in range(r0, r1):
                acc = Gt[:, r] @ v
                if r < o:
                    z[idx[ioff + r]] = acc
                else:
                    delta[doff + r - o] = acc + upd(coff + r)
    for *_, items, n_items, _ in reversed(s.levels):
        for node, r0, r1, _ in items.numpy()[:n_items]:
            ioff, o, m, _, hoff, _, _, _ = meta[node]
            Ht = H[hoff:hoff + m * o].reshape(m, o)          # H stored column-major
            w = np.array([z[idx[ioff + p]] if p < o else x[idx[ioff + p]] for p in range(m)])
            for r in range(r0, r1):
                x[idx[ioff + r]] = Ht[:, r] @ w
    return x


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("leaf", [4, 16])
def test_nested_dissection_solve_matches_sparse_lu(periodic, leaf):
    case = periodic_case(1, 4, 8, 1.0, 0.1, mesh="channel:6") if periodic else small_case(1, 4, 8, 1.0, 0.1,
                                                                                           mesh="cavity:6")
    mesh = Discretisation.build(case).mesh
    b = 6
    K = trace_pattern_matrix(mesh, b, seed=3, periodic=periodic)
    xy = mesh.nodes[mesh.face_nodes].mean(axis=1)
    s = NestedDissectionSolver(K, xy, b, device="cpu", leaf=leaf, check_tol=None)
    assert s.height > 2
    rhs = np.random.default_rng(4).standard_normal(K.shape[0])
    x = emulate_solve(s, rhs)
    ref = spsolve(K.tocsc(), rhs)
    assert np.abs(x - ref).max() <= 1e-11 * np.abs(ref).max()
    assert np.linalg.norm(K @ x - rhs) <= 1e-12 * np.linalg.norm(rhs)


def test_dissection_separates_and_covers():
    """Every face is eliminated once, and no face of one child subtree
    touches a face of its sibling's subtree (the separator cuts them)."""
    mesh = Discretisation.build(small_case(1, 4, 8, 1.0, 0.1, mesh="cavity:8")).mesh
    nf = mesh.n_faces
    rows = np.repeat(mesh.tri_faces, 3, axis=1).ravel()
    cols = np.tile(mesh.tri_faces, (1, 3)).ravel()
    A = sp.coo_matrix((np.ones(rows.size), (rows, cols)), shape=(nf, nf)).tocsr()
    A.setdiag(0)
    A.eliminate_zeros()
    A.sort_indices()
    nodes = dissect(A.indptr, A.indices, mesh.nodes[mesh.face_nodes].mean(axis=1), leaf=8)
    own = np.concatenate([n.own for n in nodes])
    assert np.array_equal(np.sort(own), np.arange(nf))

    def subtree(n):
        return np.concatenate([n.own] + [subtree(c) for c in n.children])

    for n in nodes:
        if len(n.children) == 2:
            a, c = subtree(n.children[0]), subtree(n.children[1])
            assert A[a][:, c].nnz == 0


@pytest.mark.parametrize("slots", [1216, 5])
def test_work_items_cover_every_row_once_within_shared_bounds(monkeypatch, slots):
    """Every forward row of every front (m rows of G) and every backward row
    (o rows of H) is in exactly one item of its node's height; an item holds
    at most 256 / kc rows (kc column groups of a 256-thread block, one kc per
    height, a power of two up to 64); the shared sizes passed per height cover o (forward) and m
    (backward).  Few resident blocks give whole 256-row runs at the
    wide heights, many give split columns everywhere."""
    import pbte_gb300.trace_nd as tnd
    monkeypatch.setattr(tnd, "SLOTS", slots)
    mesh = Discretisation.build(small_case(1, 4, 8, 1.0, 0.1, mesh="cavity:8")).mesh
    K = trace_pattern_matrix(mesh, 6, seed=5, periodic=False)
    xy = mesh.nodes[mesh.face_nodes].mean(axis=1)
    s = NestedDissectionSolver(K, xy, 6, device="cpu", leaf=4, check_tol=None)
    meta = s.meta.numpy()
    seen_f = [np.zeros(mt[2], dtype=int) for mt in meta]
    seen_b = [np.zeros(mt[1], dtype=int) for mt in meta]
    groups = set()
    for items_f, nf, fo, items_b, nb, bm in s.levels:
        for items, n, side in ((items_f, nf, 0), (items_b, nb, 1)):
            it = items.numpy()[:n]
            assert len(set(it[:, 3])) == 1 and it[0, 3] in tnd.GROUPS
            groups.add(int(it[0, 3]))
            for node, r0, r1, kc in it:
                assert 0 <= r0 < r1 <= meta[node][2 - side] and r1 - r0 <= tnd.THREADS // kc
                if side == 0:
                    assert meta[node][1] <= fo
                    seen_f[node][r0:r1] += 1
                else:
                    assert meta[node][2] <= bm
                    seen_b[node][r0:r1] += 1
    assert all((c == 1).all() for c in seen_f) and all((c == 1).all() for c in seen_b)
    assert (1 in groups) if slots == 5 else groups == {tnd.GROUPS[-1]}
    rhs = np.random.default_rng(6).standard_normal(K.shape[0])
    assert np.linalg.norm(K @ emulate_solve(s, rhs) - rhs) <= 1e-12 * np.linalg.norm(rhs)
