"""Host-side failure paths that need no GPU: a fabricated cyclic neighbour
graph is refused by the schedule builder with pybte's SweepCycleError
(``pybte/ordering.py:35,143-175``; pybte's own cycle tests fabricate the
graph the same way, ``tests/unit/test_ordering.py:71-112``), and the
periodic pairing refuses faces that do not line up."""
import numpy as np
import pytest

from cases import PERIODIC_EW, small_case
from pbte_gb300 import SweepCycleError
from pbte_gb300.config import Case
from pbte_gb300.discretisation import Discretisation
from pbte_gb300.sweep import direction_classes, direction_levels


def cyclic_disc():
    """The 50-triangle cavity with one shared face's normal turned around on
    one side: for every ordinate entering element 0 through that face, the
    neighbour now also sees inflow from element 0 -- a two-element cycle."""
    disc = Discretisation.build(small_case(1, 4, 8, 0.5, 0.05))
    m = disc.mesh
    il = int(np.flatnonzero(m.tri_neighbour[0] >= 0)[0])
    j = int(m.tri_neighbour[0, il])
    jl = int(np.flatnonzero(m.tri_neighbour[j] == 0)[0])
    m.tri_normal[j, jl] = m.tri_normal[0, il]
    return disc, m.tri_normal[0, il].copy()


def test_cyclic_direction_raises_sweep_cycle_error():
    disc, n0 = cyclic_disc()
    cx, cy, _ = disc.vel.flat()
    inflow = np.flatnonzero(cx * n0[0] + cy * n0[1] < 0)
    clean = np.flatnonzero(cx * n0[0] + cy * n0[1] > 0)
    assert inflow.size and clean.size
    with pytest.raises(SweepCycleError):
        direction_levels(disc, int(inflow[0]))
    # directions that never cross the turned face stay sweepable
    lv = direction_levels(disc, int(clean[0]))
    assert lv.min() >= 0
    assert direction_classes(disc).size == cx.size


def test_misaligned_periodic_pair_is_refused():
    bnds = [dict(b) for b in PERIODIC_EW]
    bnds[2]["xoff"] = -0.9            # the Master boundary no longer maps onto the Slave
    with pytest.raises(ValueError):
        Discretisation.build(Case.from_dict({
            "velmesh": {"npole": 4, "nazim": 8}, "dg": {"deg": 1},
            "flow": {"cv": 1.0, "vg": 1.0, "tau_r": 0.5, "tau_n": 0.05},
            "mesh": {"file": "channel:5:smootherstep"}, "boundaries": bnds}))
