"""Nodal Lagrange bases stored as monomial coefficients (``pybte/basis.py:31-214``).

Element basis on the reference triangle (0,0)-(1,0)-(0,1): node ``c`` sits at
``(i/deg, j/deg)`` with ``j`` the outer and ``i`` the inner loop; its shape
function is the product of the three families of Lagrange line factors.  The
monomial ``xi^a eta^b`` has index ``(a+b)(a+b+1)/2 + b`` (grouped by total
degree, then by the eta exponent), as in pybte.

Face basis on ``[-1, 1]`` with equispaced nodes ``-1 + 2i/deg``.

The coefficients are formed here by multiplying linear factors on a dense
``(deg+1, deg+1)`` coefficient grid; they equal pybte's to rounding.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

__all__ = ["Basis", "build_basis", "monomial_exponents"]


def monomial_exponents(deg: int) -> np.ndarray:
    """``(ndof, 2)`` exponents ``(a, b)`` in pybte's monomial order."""
    return np.array([(k - j, j) for k in range(deg + 1) for j in range(k + 1)],
                    dtype=np.int64)


def _mul_linear(p: np.ndarray, c0: float, cx: float, cy: float) -> np.ndarray:
    """``p(xi, eta) * (c0 + cx*xi + cy*eta)`` on a dense coefficient grid."""
    out = c0 * p
    out[1:, :] += cx * p[:-1, :]
    out[:, 1:] += cy * p[:, :-1]
    return out


def _tri_coefficients(deg: int) -> tuple[np.ndarray, np.ndarray]:
    mono = monomial_exponents(deg)
    nodes = []
    coef = []
    for j in range(deg + 1):
        for i in range(deg - j + 1):
            k = deg - i - j
            p = np.zeros((deg + 1, deg + 1))
            p[0, 0] = 1.0
            for l in range(i):          # (deg*xi - l) / (i - l)
                p = _mul_linear(p, -l / (i - l), deg / (i - l), 0.0)
            for m in range(j):          # (deg*eta - m) / (j - m)
                p = _mul_linear(p, -m / (j - m), 0.0, deg / (j - m))
            for n in range(k):          # (deg*(1-xi-eta) - n) / (k - n)
                s = 1.0 / (k - n)
                p = _mul_linear(p, (deg - n) * s, -deg * s, -deg * s)
            nodes.append((i / deg, j / deg))
            coef.append([p[a, b] for a, b in mono])
    return np.asarray(nodes), np.asarray(coef)


def _fc_coefficients(nn: int) -> tuple[np.ndarray, np.ndarray]:
    t = np.array([-1.0 + 2.0 * i / (nn - 1) for i in range(nn)])
    coef = np.zeros((nn, nn))
    for i in range(nn):
        p = np.zeros(nn)
        p[0] = 1.0
        for j in range(nn):
            if j == i:
                continue
            d = t[i] - t[j]
            q = np.zeros(nn)
            q[1:] = p[:-1] / d
            q -= p * (t[j] / d)
            p = q
        coef[i] = p
    return t, coef


@dataclass(frozen=True)
class Basis:
    deg: int
    node_fc: np.ndarray        # (ndof_fc,)
    nodfun_fc: np.ndarray      # (ndof_fc, ndof_fc): phi_i(t) = sum_k c[i,k] t^k
    node_tri: np.ndarray       # (ndof_tri, 2)
    nodfun_tri: np.ndarray     # (ndof_tri, ndof_tri): over monomials
    mono: np.ndarray           # (ndof_tri, 2)

    @property
    def ndof_tri(self) -> int:
        return self.nodfun_tri.shape[0]

    @property
    def ndof_fc(self) -> int:
        return self.nodfun_fc.shape[0]

    def eval_tri(self, xi, eta) -> np.ndarray:
        """Every shape function at the points ``(xi, eta)``: shape (..., ndof)."""
        xi = np.asarray(xi, dtype=np.float64)
        eta = np.asarray(eta, dtype=np.float64)
        out = np.zeros(np.broadcast(xi, eta).shape + (self.ndof_tri,))
        for k, (a, b) in enumerate(self.mono):
            out += self.nodfun_tri[:, k] * (xi ** float(a) * eta ** float(b))[..., None]
        return out

    def eval_fc(self, t) -> np.ndarray:
        t = np.asarray(t, dtype=np.float64)
        out = np.zeros(t.shape + (self.ndof_fc,))
        for k in range(self.ndof_fc):
            out += self.nodfun_fc[:, k] * (t ** float(k))[..., None]
        return out


def build_basis(deg: int) -> Basis:
    if deg < 1:
        raise ValueError("deg >= 1 required")
    node_tri, nodfun_tri = _tri_coefficients(deg)
    node_fc, nodfun_fc = _fc_coefficients(deg + 1)
    return Basis(deg=deg, node_fc=node_fc, nodfun_fc=nodfun_fc, node_tri=node_tri,
                 nodfun_tri=nodfun_tri, mono=monomial_exponents(deg))
