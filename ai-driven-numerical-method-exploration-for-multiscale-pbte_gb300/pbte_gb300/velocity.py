"""Discrete ordinates (``pybte/velocity.py:59-86``).

Polar angle ``the`` (measured from the x axis) takes the Gauss-Legendre
nodes on ``[0, pi]`` with the rule's descending order reversed (so
ascending); azimuth ``phi`` takes the nodes on ``[0, pi]`` then on
``[pi, 2 pi]``, each half reversed the same way.  With
``cx = vg cos(the)``, ``cy = vg sin(the) cos(phi)`` and
``domega = sin(the) w_the w_phi`` (summing to 4 pi), directions are flattened
as ``d = j1 + npole * j2`` (pole fastest).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .constants import PI
from .quadrature import gauss_legendre

__all__ = ["VelocityMesh", "build_velocity_mesh", "twin_map"]


@dataclass(frozen=True)
class VelocityMesh:
    the: np.ndarray
    wthe: np.ndarray
    phi: np.ndarray
    wphi: np.ndarray
    domega: np.ndarray   # (npole, nazim)
    cx: np.ndarray
    cy: np.ndarray

    @property
    def npole(self) -> int:
        return self.the.size

    @property
    def nazim(self) -> int:
        return self.phi.size

    @property
    def ndir(self) -> int:
        return self.npole * self.nazim

    def flat(self):
        return (self.cx.ravel(order="F"), self.cy.ravel(order="F"),
                self.domega.ravel(order="F"))


def build_velocity_mesh(npole: int, nazim: int, vg: float = 1.0) -> VelocityMesh:
    nazim = (nazim // 2) * 2
    if nazim < 2 or npole < 1:
        raise ValueError("need npole >= 1 and nazim >= 2")
    half = nazim // 2
    a, w = gauss_legendre(npole, 0.0, PI)
    the, wthe = a[::-1].copy(), w[::-1].copy()
    a1, w1 = gauss_legendre(half, 0.0, PI)
    a2, w2 = gauss_legendre(half, PI, 2.0 * PI)
    phi = np.concatenate([a1[::-1], a2[::-1]])
    wphi = np.concatenate([w1[::-1], w2[::-1]])
    if half == 1:
        raise ValueError("nazim >= 4 required (a one-point azimuth rule has no Newton start)")
    st = np.sin(the)
    domega = (st * wthe)[:, None] * wphi[None, :]
    cx = np.repeat((vg * np.cos(the))[:, None], nazim, axis=1)
    cy = (vg * st)[:, None] * np.cos(phi)[None, :]
    return VelocityMesh(the=the, wthe=wthe, phi=phi, wphi=wphi, domega=domega, cx=cx, cy=cy)


def twin_map(cxv: np.ndarray, cyv: np.ndarray, domega: np.ndarray,
             tol: float = 1e-12) -> np.ndarray:
    """For each direction the index of its z-mirror twin (same in-plane
    velocity and weight, ``cz -> -cz``), or itself when it has none.

    In a 2D problem a direction and its z-mirror see identical transport, so
    their distributions coincide; the GPU path sweeps one of each pair."""
    n = cxv.size
    twin = np.arange(n)
    used = np.zeros(n, dtype=bool)
    for d in range(n):
        if used[d]:
            continue
        cand = np.flatnonzero((~used) & (np.arange(n) != d)
                              & (np.abs(cxv - cxv[d]) <= tol)
                              & (np.abs(cyv - cyv[d]) <= tol)
                              & (np.abs(domega - domega[d]) <= tol * max(1.0, abs(domega[d]))))
        used[d] = True
        if cand.size:
            twin[d] = cand[0]
            twin[cand[0]] = d
            used[cand[0]] = True
    return twin
