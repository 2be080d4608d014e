"""Device solve of the GSIS trace system ``K x = b``
(``pybte/acceleration/global_solve.py:120-195``, where pybte factorises
``K`` once with SuperLU and runs its two triangular solves every iteration).

``K`` has one dense ``b x b`` block (``b = 3 (deg + 1)``) for every pair of
faces that share an element, and depends only on the geometry and the
relaxation times, so it is factorised once, by nested dissection:

* Ordering (host).  The faces are split recursively along the longer side
  of their midpoints' box at the median; the faces of the left half that
  touch the right half form the separator.  Every face is eliminated before
  the faces of the separators above it (a post-order of the dissection
  tree).
* Multifrontal factorisation (device, dense library calls at setup).  A
  tree node's *front* holds its own faces (fully summed) and its boundary
  faces (neighbours eliminated later).  The front is assembled from the
  blocks of ``K`` whose earlier-eliminated face is one of the node's own
  (each block exactly once) plus its children's update matrices
  (extend-add), then partially factorised: ``P F11 = L11 U11`` (partial
  pivoting within the own faces), ``U12 = L11^-1 P F12``,
  ``L21 = F21 U11^-1``, and ``F22 - L21 U12`` goes to the parent.
* Solve operators.  The triangular factors are inverted once, so each
  node's forward and backward steps are dense matrix-vector products:
  ``G = [L11^-1 P ; -L21 L11^-1 P]`` maps the node's own right-hand side to
  its forward values and the update of its boundary, and
  ``H = [U11^-1, -U11^-1 U12]`` maps ``[forward values, x of the boundary]``
  to the node's unknowns.  Both are stored column-major, so that the solve
  kernels give each output row a thread and read the rows of a column
  coalesced.

The solve (``pbte_nd_forward`` / ``pbte_nd_backward``) walks the tree by
height, one launch per height and direction, over work items of a front's
rows and a count of column groups; a node's right-hand side adds its
children's updates in a fixed order and the column groups' partial sums
are added by a fixed tree, so the result is deterministic.
At setup the device solve of a random right-hand side is checked against
``K`` (relative residual below ``check_tol``).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib

__all__ = ["NestedDissectionSolver", "dissect"]

#: threads per block of the solve kernels, and the work items aimed at per
#: tree height (measured on GB300, solve at 8192 / 32768 triangles P2:
#: 608 items 0.414 / 1.15 ms, 912 0.426 / 1.19, 1216 0.435 / 1.19)
THREADS = 256
SLOTS = 608
#: column-group counts a height may use (a power of two, at most 64)
GROUPS = (1, 2, 4, 8, 16, 32, 64)


def _ranges(ptr: np.ndarray, rows: np.ndarray):
    """CSR entries of ``rows``: (owning position in ``rows``, entry index)."""
    starts = ptr[rows]
    lens = ptr[rows + 1] - starts
    total = int(lens.sum())
    owner = np.repeat(np.arange(rows.size), lens)
    first = np.repeat(np.cumsum(lens) - lens, lens)
    return owner, np.repeat(starts, lens) + (np.arange(total) - first)


class _Node:
    __slots__ = ("own", "children", "parent", "height", "bnd")

    def __init__(self, own, children):
        self.own = own
        self.children = children
        self.parent = None
        self.height = 0
        self.bnd = None


def dissect(adj_ptr: np.ndarray, adj: np.ndarray, xy: np.ndarray, leaf: int = 32) -> list:
    """Nested-dissection tree of a graph with vertex coordinates ``xy``
    (CSR adjacency ``adj_ptr``/``adj``, no self loops); the nodes in
    post-order (children first)."""
    side = np.zeros(xy.shape[0], dtype=np.int8)     # scratch: 1 left, 2 right
    order = []

    def build(S):
        if S.size <= leaf:
            node = _Node(S, [])
            order.append(node)
            return node
        ext = xy[S].max(axis=0) - xy[S].min(axis=0)
        srt = S[np.argsort(xy[S, int(np.argmax(ext))], kind="stable")]
        left, right = srt[:srt.size // 2], srt[srt.size // 2:]
        side[left] = 1
        side[right] = 2
        owner, ent = _ranges(adj_ptr, left)
        touches = np.zeros(left.size, dtype=bool)
        touches[owner[side[adj[ent]] == 2]] = True
        side[left] = 0
        side[right] = 0
        kids = [build(np.sort(p)) for p in (left[~touches], right) if p.size]
        node = _Node(np.sort(left[touches]), kids)
        for k in kids:
            k.parent = node
        order.append(node)
        return node

    build(np.arange(xy.shape[0]))
    return order


_LINALG = {}


def _linalg_device(dev: torch.device) -> torch.device:
    """``dev`` if torch's dense factorisation runs there (its CUDA linear
    algebra is a separately loaded library), else the host."""
    if dev.type != "cuda":
        return dev
    if dev not in _LINALG:
        try:
            torch.linalg.lu_factor(torch.eye(2, dtype=torch.float64, device=dev))
            _LINALG[dev] = dev
        except RuntimeError:
            _LINALG[dev] = torch.device("cpu")
    return _LINALG[dev]


class NestedDissectionSolver:
    """``solve(b) -> x`` for the trace matrix ``K`` (scipy sparse, face-major
    blocks of size ``block``: unknown ``f * block + c``), on ``device``."""

    def __init__(self, K, face_xy: np.ndarray, block: int, device, leaf: int = 32,
                 check_tol: float | None = 1e-10):
        K = sp.csr_matrix(K)
        n_faces = face_xy.shape[0]
        b = int(block)
        if K.shape != (n_faces * b, n_faces * b):
            raise ValueError("K does not have one block per face")
        self.device = torch.device(device)
        self.n = K.shape[0]
        self.block = b
        Kb = sp.bsr_matrix(K, blocksize=(b, b))
        Kb.sort_indices()
        KT = Kb.transpose().tobsr(blocksize=(b, b))
        KT.sort_indices()
        rows = np.repeat(np.arange(n_faces), np.diff(Kb.indptr))
        A = sp.coo_matrix((np.ones(rows.size), (rows, Kb.indices)), shape=(n_faces, n_faces)).tocsr()
        A = (A + A.T).tocsr()
        A.setdiag(0)
        A.eliminate_zeros()
        A.sort_indices()
        nodes = dissect(A.indptr, A.indices, np.asarray(face_xy, dtype=np.float64), leaf)
        pos = np.empty(n_faces, dtype=np.int64)
        ends = []
        k = 0
        for nd in nodes:
            pos[nd.own] = np.arange(k, k + nd.own.size)
            k += nd.own.size
            ends.append(k)
        for nd, k in zip(nodes, ends):
            # boundary: neighbours of the own faces and the children's
            # boundaries eliminated after this subtree
            _, ent = _ranges(A.indptr, nd.own)
            cand = np.unique(np.concatenate([A.indices[ent]] + [c.bnd for c in nd.children]))
            nd.bnd = cand[pos[cand] >= k] if cand.size else cand
            nd.height = 1 + max((c.height for c in nd.children), default=-1)
        self.n_nodes = len(nodes)
        self.height = max(nd.height for nd in nodes) + 1
        self._layout(nodes, b)
        self._factor(nodes, Kb, KT, b)
        self.check_residual = self._check(K, check_tol) if check_tol is not None else None

    # -- device layout -------------------------------------------------------
    def _layout(self, nodes, b):
        dev = self.device
        n_faces = self.n // b
        N = len(nodes)

        def starts(v):                                   # exclusive prefix sums
            out = np.zeros(v.size, dtype=np.int64)
            np.cumsum(v[:-1], out=out[1:])
            return out

        own_n = np.array([nd.own.size for nd in nodes], dtype=np.int64)
        fn = own_n + np.array([nd.bnd.size for nd in nodes], dtype=np.int64)   # faces per front
        o, m = own_n * b, fn * b
        i_off, g_off, d_off, c_off = starts(m), starts(m * o), starts(m - o), starts(m + 1)
        faces = np.concatenate([f for nd in nodes for f in (nd.own, nd.bnd)]).astype(np.int64)
        # the children's boundary updates: child boundary face -> its position
        # in the parent's front (a sorted (node, face) key), by front position
        # with the children in order
        at = {id(nd): i for i, nd in enumerate(nodes)}
        par = np.array([i for i, nd in enumerate(nodes) for _ in nd.children], dtype=np.int64)
        kid = np.array([at[id(ch)] for nd in nodes for ch in nd.children], dtype=np.int64)
        if kid.size:
            kb = fn[kid] - own_n[kid]                    # boundary faces of each child
            key = np.repeat(np.arange(N, dtype=np.int64), fn) * n_faces + faces
            order = np.argsort(key, kind="stable")
            q = np.repeat(par, kb) * n_faces + np.concatenate([nodes[k].bnd for k in kid]).astype(np.int64)
            pos = order[np.searchsorted(key[order], q)] - np.repeat(starts(fn)[par], kb)
            tgt = (pos[:, None] * b + np.arange(b)).ravel()
            nb = kb * b
            src = np.repeat(d_off[kid], nb) + (np.arange(nb.sum()) - np.repeat(starts(nb), nb))
            gkey = np.repeat(i_off[par], nb) + tgt                 # position over all fronts
            srt = np.argsort(gkey, kind="stable")
            csrc = src[srt]
            counts = np.bincount(gkey, minlength=int(m.sum()))
        else:
            csrc = np.zeros(0, dtype=np.int64)
            counts = np.zeros(int(m.sum()), dtype=np.int64)
        cum = np.zeros(counts.size + 1, dtype=np.int64)
        np.cumsum(counts, out=cum[1:])
        n_ptr = int((m + 1).sum())
        cptr = cum[np.repeat(i_off, m + 1) + (np.arange(n_ptr) - np.repeat(c_off, m + 1))]
        meta = np.stack([i_off, o, m, g_off, g_off, d_off, c_off, np.zeros(N, dtype=np.int64)], axis=1)
        idx = (faces[:, None] * b + np.arange(b)).ravel()
        g_total = int((m * o).sum())
        d_total = int((m - o).sum())
        # work items (node, first row, end row, column groups kc): a block
        # of 256 threads holds 256 / kc rows, a thread per row and column
        # group.  Per height the smallest kc of GROUPS that gives at least
        # SLOTS items, so the few long-row fronts near the root split their
        # columns over more SMs; a node's rows are cut into even runs.
        rows = np.stack([m, o], axis=1)                                    # forward m, backward o
        h_of = np.array([nd.height for nd in nodes])

        def pieces(r, kc):
            return -(-r // (THREADS // kc))

        def cuts(sel, r, kc):
            # each node's rows cut into n even runs, at round(i * r / n) (the
            # points of numpy's linspace(0, r, n + 1))
            n = pieces(r, kc)
            node = np.repeat(sel, n)
            i = np.arange(n.sum()) - np.repeat(starts(n), n)
            step = np.repeat(r / np.maximum(n, 1), n)
            first = np.round(i * step).astype(np.int64)
            last = np.where(i + 1 == np.repeat(n, n), np.repeat(r, n), np.round((i + 1) * step).astype(np.int64))
            keep = last > first
            items = np.stack([node, first, last, np.full(node.size, kc)], axis=1)[keep]
            return items.astype(np.int32)

        self.levels = []
        empty = torch.zeros((1, 4), dtype=torch.int32, device=dev)
        for h in range(self.height):
            sel = np.flatnonzero(h_of == h)
            lv = []
            for side, width in ((0, o), (1, m)):
                r = rows[sel, side]
                kc = next((k for k in GROUPS if pieces(r, k).sum() >= SLOTS), GROUPS[-1])
                items = cuts(sel, r, kc)
                # shared memory: the largest o (forward) / m (backward) of the items' nodes
                big = int(width[np.unique(items[:, 0])].max()) if len(items) else 0
                lv.append((torch.from_numpy(items).to(dev) if len(items) else empty, len(items), big))
            (fi, nf_, fo), (bi, nb_, bm) = lv
            self.levels.append((fi, nf_, fo, bi, nb_, bm))
        f64 = dict(dtype=torch.float64, device=dev)
        self.meta_host = np.ascontiguousarray(meta, dtype=np.int64)
        self.meta = torch.from_numpy(self.meta_host).to(dev)
        self.idx = torch.from_numpy(idx.astype(np.int32)).to(dev)
        self.cptr = torch.from_numpy(cptr).to(dev)
        self.csrc = torch.from_numpy(np.concatenate([csrc, np.zeros(1, np.int64)])).to(dev)
        self.Gd = torch.empty(max(g_total, 1), **f64)
        self.Hd = torch.empty(max(g_total, 1), **f64)
        self.factor_entries = 2 * g_total
        self.max_front = int(m.max())
        self.z = torch.zeros(self.n, **f64)
        self.delta = torch.zeros(max(d_total, 1), **f64)

    # -- factorisation -----------------------------------------------------------
    #: fronts factorised together: at most this many, and padded to at most
    #: this factor of the smallest front of the batch
    BATCH_FRONTS = 512
    BATCH_PAD = 1.3

    def _factor(self, nodes, Kb, KT, b):
        """Fronts assembled and factorised on ``self.device`` (or on the host
        where the device's dense linear-algebra library cannot be loaded); G
        and H written into their slices of ``Gd`` / ``Hd``.

        The fronts of one tree height are independent, so they are processed
        in batches of similar size: each front is padded to the batch's
        largest own and boundary parts (own faces first, padded with an
        identity block; boundary faces after the batch's own part, padded
        with zeros), so one batched LU with partial pivoting and a handful of
        batched products do the work of a front each.  The padding neither
        changes the pivots (a padding row is zero in every real column) nor
        the real blocks of G, H and the update passed to the parent."""
        dst = self.device
        dev = _linalg_device(dst)
        f64 = dict(dtype=torch.float64, device=dev)
        n_faces = Kb.shape[0] // b
        kb_data = torch.from_numpy(np.ascontiguousarray(Kb.data)).to(dev)
        kt_data = torch.from_numpy(np.ascontiguousarray(np.transpose(KT.data, (0, 2, 1)))).to(dev)
        meta = {id(nd): self.meta_host[i] for i, nd in enumerate(nodes)}
        upd = {}
        by_height = {}
        for nd in nodes:
            by_height.setdefault(nd.height, []).append(nd)
        loc = np.full(n_faces, -1, dtype=np.int64)
        for h in sorted(by_height):
            group = sorted(by_height[h], key=lambda nd: nd.own.size + nd.bnd.size)
            start = 0
            while start < len(group):
                m0 = max(1, group[start].own.size + group[start].bnd.size)
                stop = start + 1
                while (stop < len(group) and stop - start < self.BATCH_FRONTS
                       and group[stop].own.size + group[stop].bnd.size <= self.BATCH_PAD * m0):
                    stop += 1
                self._factor_batch(group[start:stop], Kb, KT, kb_data, kt_data, b, loc, upd, meta, dev, f64)
                start = stop

    def _factor_batch(self, batch, Kb, KT, kb_data, kt_data, b, loc, upd, meta, dev, f64):
        dst = self.device
        B = len(batch)
        NO = max(nd.own.size for nd in batch)          # padded own faces
        NB = max(nd.bnd.size for nd in batch)          # padded boundary faces
        MF = NO + NB
        F = torch.zeros((B, MF, MF, b, b), **f64)      # block (front face, front face) of every front
        kb_b, kb_r, kb_c, kb_e = [], [], [], []
        kt_b, kt_r, kt_c, kt_e = [], [], [], []
        ch_b, ch_r, ch_c, ch_v = [], [], [], []
        for k, nd in enumerate(batch):
            no = nd.own.size
            loc[nd.own] = np.arange(no)
            loc[nd.bnd] = NO + np.arange(nd.bnd.size)
            if no:
                # blocks K[own, front] from the rows, K[bnd, own] from the columns
                owner, ent = _ranges(Kb.indptr, nd.own)
                c = loc[Kb.indices[ent]]
                keep = np.flatnonzero(c >= 0)
                kb_b.append(np.full(keep.size, k)), kb_r.append(owner[keep]), kb_c.append(c[keep])
                kb_e.append(ent[keep])
                owner, ent = _ranges(KT.indptr, nd.own)
                c = loc[KT.indices[ent]]
                keep = np.flatnonzero(c >= NO)
                kt_b.append(np.full(keep.size, k)), kt_r.append(c[keep]), kt_c.append(owner[keep])
                kt_e.append(ent[keep])
            for ch in nd.children:
                S = upd.pop(id(ch))
                L = ch.bnd.size
                kp = loc[ch.bnd]
                ch_b.append(np.full(L * L, k))
                ch_r.append(np.repeat(kp, L))
                ch_c.append(np.tile(kp, L))
                ch_v.append(S.view(L, b, L, b).permute(0, 2, 1, 3).reshape(L * L, b, b))
            loc[nd.own] = -1
            loc[nd.bnd] = -1
        T = lambda parts: torch.from_numpy(np.concatenate(parts)).to(dev)   # noqa: E731
        if kb_b:
            F.index_put_((T(kb_b), T(kb_r), T(kb_c)), kb_data[T(kb_e)], accumulate=True)
            F.index_put_((T(kt_b), T(kt_r), T(kt_c)), kt_data[T(kt_e)], accumulate=True)
        if ch_b:
            F.index_put_((T(ch_b), T(ch_r), T(ch_c)), torch.cat(ch_v), accumulate=True)
        # identity blocks on the padded own faces, all fronts at once
        pad_k = np.concatenate([np.full(NO - nd.own.size, k) for k, nd in enumerate(batch)])
        if pad_k.size:
            pad_p = np.concatenate([np.arange(nd.own.size, NO) for nd in batch])
            F[T([pad_k]), T([pad_p]), T([pad_p])] = torch.eye(b, **f64)
        Fm = F.permute(0, 1, 3, 2, 4).reshape(B, MF * b, MF * b)
        del F
        o_, m_ = NO * b, MF * b
        F11, F12, F21, F22 = Fm[:, :o_, :o_], Fm[:, :o_, o_:], Fm[:, o_:, :o_], Fm[:, o_:, o_:]
        if o_:
            LU, piv = torch.linalg.lu_factor(F11)
            P, Lf, Uf = torch.lu_unpack(LU, piv)
            eye = torch.eye(o_, **f64).expand(B, o_, o_)
            Linv = torch.linalg.solve_triangular(Lf, eye, upper=False, unitriangular=True)
            Uinv = torch.linalg.solve_triangular(Uf, eye, upper=True)
            # L11^-1 P^T: P^T permutes the columns of L11^-1 (column j is
            # column sigma(j), sigma(j) the column of row j's one in P)
            sigma = P.argmax(dim=-1)
            Gtop = torch.gather(Linv, 2, sigma[:, None, :].expand(B, o_, o_))
            U12 = Gtop @ F12
            L21 = F21 @ Uinv
            S = F22 - L21 @ U12
            Gbot = -(L21 @ Gtop)
            Hr = -(Uinv @ U12)
        else:
            S = F22.clone()
        mt = np.array([meta[id(nd)][:5] for nd in batch], dtype=np.int64)
        if o_:
            # G^T (o x m) and H^T (m x o) of every front, column-major, out of
            # the padded batch in one gather and one scatter each: front
            # row r < o is padded row r, boundary row r >= o padded row
            # o_ + r - o
            Gfull = torch.cat([Gtop, Gbot], dim=1)                        # (B, m_, o_): G rows
            Hfull = torch.cat([Uinv, Hr], dim=2)                          # (B, o_, m_): H rows
            self._scatter_columns(Gfull, mt[:, 1], mt[:, 2], mt[:, 3], o_, True, self.Gd, dev)
            self._scatter_columns(Hfull, mt[:, 1], mt[:, 2], mt[:, 4], o_, False, self.Hd, dev)
            del Gfull, Hfull
        for k, nd in enumerate(batch):
            if nd.parent is not None:
                mb = int(mt[k, 2] - mt[k, 1])
                upd[id(nd)] = S[k, :mb, :mb]

    @staticmethod
    def _scatter_columns(full, o, m, off, o_, is_g, out, dev):
        """Write each front's factor column-major into ``out``: G^T[c][r] =
        G[r][c] at ``off + c * m + r`` (``is_g``; ``full`` (B, m_, o_)), or
        H^T[r][c] = H[c][r] at ``off + r * o + c`` (``full`` (B, o_, m_))."""
        size = o * m
        keep = np.flatnonzero(size > 0)
        if not keep.size:
            return
        starts = np.zeros(keep.size + 1, dtype=np.int64)
        np.cumsum(size[keep], out=starts[1:])
        total = int(starts[-1])
        i64 = dict(dtype=torch.int64, device=dev)
        t = torch.arange(total, **i64)
        k = torch.searchsorted(torch.from_numpy(starts[1:]).to(dev), t, right=True)
        l = t - torch.from_numpy(starts[:-1]).to(dev)[k]
        ok = torch.from_numpy(o[keep]).to(dev)[k]
        mk = torch.from_numpy(m[keep]).to(dev)[k]
        kb = torch.from_numpy(keep).to(dev)[k]
        dst = torch.from_numpy(off[keep]).to(dev)[k] + l
        if is_g:
            c, r = l // mk, l % mk
        else:
            r, c = l // ok, l % ok
        rs = torch.where(r < ok, r, o_ + r - ok)          # the padded front row of front row r
        B, d1, d2 = full.shape
        if is_g:
            src = (kb * d1 + rs) * d2 + c                  # full[kb, rs, c]
        else:
            src = (kb * d1 + c) * d2 + rs                  # full[kb, c, rs]
        vals = full.reshape(-1)[src]
        out[dst.to(out.device)] = vals.to(out.device)

    # -- solve -----------------------------------------------------------------
    def solve(self, b: torch.Tensor, out: torch.Tensor | None = None, stream=None, done=None) -> torch.Tensor:
        """``K^-1 b`` on the device (``b``: float64, n entries); into ``out``
        when given, else a new tensor.  ``done``: an int32 device flag that
        makes every launch return at once while it is nonzero."""
        if self.device.type != "cuda":
            raise RuntimeError("the trace solve runs on the GPU; there is no CPU fallback")
        L = _lib.lib()
        s = (stream or torch.cuda.current_stream(self.device)).cuda_stream
        b = b.contiguous()
        x = out if out is not None else torch.empty(self.n, dtype=torch.float64, device=self.device)
        for items, n_items, fo, _, _, _ in self.levels:
            if n_items:
                _lib.check(L.pbte_nd_forward(items.data_ptr(), n_items, self.meta.data_ptr(), self.idx.data_ptr(),
                                             self.cptr.data_ptr(), self.csrc.data_ptr(), self.Gd.data_ptr(),
                                             b.data_ptr(), self.z.data_ptr(), self.delta.data_ptr(), fo,
                                             None if done is None else done.data_ptr(), s),
                           "nd_forward")
        for _, _, _, items, n_items, bm in reversed(self.levels):
            if n_items:
                _lib.check(L.pbte_nd_backward(items.data_ptr(), n_items, self.meta.data_ptr(), self.idx.data_ptr(),
                                              self.Hd.data_ptr(), self.z.data_ptr(), x.data_ptr(), bm,
                                              None if done is None else done.data_ptr(), s),
                           "nd_backward")
        return x

    def _check(self, K, tol) -> float:
        rng = np.random.default_rng(0)
        rhs = K @ rng.standard_normal(self.n)
        x = self.solve(torch.from_numpy(rhs).to(self.device)).cpu().numpy()
        res = float(np.linalg.norm(K @ x - rhs) / max(np.linalg.norm(rhs), 1e-300))
        if not res < tol:
            raise np.linalg.LinAlgError(f"nested-dissection trace solve: relative residual {res:.2e} > {tol:.0e}")
        return res
