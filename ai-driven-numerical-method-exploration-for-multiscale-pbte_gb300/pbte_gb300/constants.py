"""Physical/boundary constants; the codes and tables of ``pybte/constants.py:11-49``."""
from __future__ import annotations

import math

#: pybte's PI is 4*atan(1) in double precision, i.e. math.pi
PI: float = 4.0 * math.atan(1.0)

BC_THERMALISING = 1      # isothermal, diffusely emitting wall
BC_NONTHERMALISING = 2   # adiabatic, diffusely reflecting wall
BC_PERIODIC = 3          # periodic pair
BC_SYMMETRY = 4          # rejected, as pybte does

BC_TYPE_NAMES = {
    "thermalising": BC_THERMALISING, "thermalizing": BC_THERMALISING,
    "isothermal": BC_THERMALISING,
    "nonthermalising": BC_NONTHERMALISING, "nonthermalizing": BC_NONTHERMALISING,
    "adiabatic": BC_NONTHERMALISING,
    "periodic": BC_PERIODIC, "symmetry": BC_SYMMETRY,
}

#: number of element quadrature points per degree (pybte's NP_TRI table)
NP_TRI_BY_DEG = {1: 3, 2: 6, 3: 12, 4: 16}
#: points of the Gauss-Legendre face rule used for the numerical face tensors
NP_FC_DEFAULT = 15
