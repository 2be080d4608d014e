"""pbte_gb300 -- GB300-native (sm_103a) steady gray linearised-Callaway DG
discrete-ordinates solver, a drop-in for the hot path of pybte
(dingtao-shen/AI-Driven-Numerical-Method-Exploration-for-Multiscale-PBTE,
``solver-python/pybte``): the transport sweep and the CIS / GMRES / GSIS
outer iterations run as hand-written CUDA kernels behind pybte's
``Case`` / ``Solver`` / ``SweepContext`` interface.

>>> from pbte_gb300 import Case, Solver
>>> rec = Solver(case).run()
"""
from .config import Case, square_case
from .discretisation import Discretisation

__all__ = ["Case", "square_case", "Discretisation", "Solver", "SweepContext", "Moments",
           "RunRecord", "SweepCycleError", "build"]


def build(force: bool = False):
    from ._lib import build as _build
    return _build(force=force)


def __getattr__(name):
    if name in ("Solver", "RunRecord"):
        from . import solver
        return getattr(solver, name)
    if name in ("SweepContext", "Moments", "SweepCycleError"):
        from . import sweep
        return getattr(sweep, name)
    raise AttributeError(name)
