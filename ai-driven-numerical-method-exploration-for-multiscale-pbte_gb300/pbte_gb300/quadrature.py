"""Gauss-Legendre rules, restating ``pybte/quadrature.py:242-304``.

pybte transcribes a Fortran Newton iteration: a perturbed-cosine start, the
three-term Legendre recurrence, a stop when the Newton step is under 1e-13,
and weights formed from the derivative taken at the *previous* iterate.  The
last detail moves the weights by ~1e-13 relative to exact Gauss weights, and
the discrete ordinates are built on these weights, so the same iteration is
followed here to give the same ordinates bit for bit.  Nodes come out in
descending order, as pybte's do.
"""
from __future__ import annotations

import numpy as np

from .constants import PI

__all__ = ["gl_core", "gauss_legendre", "face_rule"]

_CACHE: dict[int, tuple[np.ndarray, np.ndarray]] = {}


def gl_core(n: int, tol: float = 1.0e-13, max_sweeps: int = 200):
    """``(y, lp)``: descending nodes on [-1, 1] and the scaled derivative."""
    if n < 2:
        raise ValueError("the Newton start divides by (n - 1); n >= 2 required")
    if n in _CACHE:
        return _CACHE[n]
    i = np.arange(1, n + 1, dtype=np.float64)
    y = (np.cos((2.0 * (i - 1.0) + 1.0) * PI / (2.0 * (n - 1.0) + 2.0))
         + 0.27 / n * np.sin(PI * (-1.0 + i * 2.0 / (n - 1.0)) * (n - 1.0) / (n + 1)))
    for _ in range(max_sweeps):
        pkm1 = np.ones(n)
        pk = y.copy()
        for k in range(2, n + 1):
            pkm1, pk = pk, ((2.0 * k - 1.0) * y * pk - (k - 1) * pkm1) / k
        # pk = P_n(y), pkm1 = P_{n-1}(y); lp = (n+1)/n * P_n'(y)
        lp = (n + 1) * (pkm1 - y * pk) / (1.0 - y * y)
        y_prev = y
        y = y_prev - pk / lp
        if np.max(np.abs(y - y_prev)) < tol:
            break
    else:
        raise RuntimeError("Gauss-Legendre iteration did not converge")
    _CACHE[n] = (y, lp)
    return y, lp


def gauss_legendre(n: int, a: float, b: float):
    """Abscissae (descending) and weights of the ``n``-point rule on ``[a, b]``."""
    y, lp = gl_core(n)
    absc = (a * (1.0 - y) + b * (1.0 + y)) / 2.0
    weig = (n + 1) * (n + 1) * (b - a) / ((1.0 - y * y) * lp * lp) / n / n
    return absc, weig


def face_rule(n: int, length: np.ndarray):
    """One rule per face on ``[0, length]``: ``(absc, weig)`` of shape (k, n)."""
    y, lp = gl_core(n)
    L = np.asarray(length, dtype=np.float64)[:, None]
    absc = (0.0 * (1.0 - y) + L * (1.0 + y)) / 2.0
    weig = (n + 1) * (n + 1) * (L - 0.0) / ((1.0 - y * y) * lp * lp) / n / n
    return absc, weig
