"""The oracle's water loop with molecular cells against the reference's own event loop (CPU; no reference tree).

``tests/golden/make_water_cell_trajectories.py`` recorded the reference's ``SingleProcessMediator.run`` on flexible
water with the molecular cells of its water cell-veto configuration: root units in ``SingleActiveCellOccupancy``,
the summed-bounding Coulomb factor with the molecules of the nearby cells and the surplus molecules, the molecular
cell veto (``CompositeObjectCellVetoEventHandler`` with the ``DipoleMonteCarloEstimator``'s bound tables, stored with
the trajectory) and the cell-boundary events of the active root unit, which keep the bond and Lennard-Jones
candidates alive.  The oracle (``oracle/jf_oracle.c``: ``jfo_water_cells_create``, ``water_cells_run``) replays every
event from the same initial state and keyed random numbers.

Four trajectories are reproduced bit for bit (every logged field, the root of the moved unit's molecule after every
event, the final leaf and root positions): two with the molecular cell veto and two with the molecular cell-bounding
far field of the reference's dipole configuration (``TwoCompositeObjectCellBoundingPotentialEventHandler``, a factor
for every occupied far cell).  ``water_n8_cell_boundaries`` runs 5000 events with 81 cell boundaries, 63 of them followed by a bond or Lennard-Jones event that commits the in-state copies of its creation;
it is bit for bit up to event 3699, whose H-H bond solve squares 1.0750481431014438: CPython's ``**`` calls the C
library's ``pow``, which returns 1.1557285099858623 there, one unit in the last place below the correctly rounded
square 1.1557285099858625 that the oracle (and the GPU) compute.  From there on every discrete field still matches
and the event times stay within 1e-14 relative.
"""
import json

import numpy as np
import pytest

import oracle

GOLDEN = "tests/golden/%s.npz"
DISCRETE = ("kind", "moved", "target", "new_active", "new_direction", "accepted")


def load(name):
    z = np.load(GOLDEN % name)
    spec = json.loads(str(z["spec"]))
    return z, spec


def run_oracle(z, spec, events=None):
    system = oracle.make_water_system(spec, spec["rng_key"])
    water = oracle.Water(system, z["initial"], z["charges"],
                         cells=(spec["cells_per_side"], spec["neighbor_layers"], z["initial_roots"],
                                z["bounds_upper"], z["bounds_lower"], True, spec.get("far", "cell_veto"),
                                spec["dipole_charge"]))
    log, roots = water.run(len(z["events"]) if events is None else events, roots=True)
    return water, log, roots


@pytest.mark.parametrize("name", ["water_n8_cell_veto", "water_n64_cell_veto", "water_n8_cell_bounding",
                                  "water_n64_cell_bounding"])
def test_trajectory_bit_for_bit(name):
    z, spec = load(name)
    water, log, roots = run_oracle(z, spec)
    ref = z["events"]
    assert len(log) == len(ref)
    assert log.tobytes() == ref.tobytes()
    assert np.array_equal(roots, z["roots"])
    assert np.array_equal(water.positions(), z["final"])
    assert np.array_equal(water.roots(), z["final_roots"])


def test_cell_boundaries_and_persistent_pairs():
    z, spec = load("water_n8_cell_boundaries")
    ref = z["events"]
    boundaries = np.nonzero(ref["kind"] == oracle.EV_BOUNDARY)[0]
    following = ref["kind"][boundaries[boundaries + 1 < len(ref)] + 1]
    assert len(boundaries) >= 50
    assert np.sum((following == oracle.EV_BOND) | (following == oracle.EV_PAIR)) >= 40
    water, log, roots = run_oracle(z, spec)
    first_inexact = next(i for i in range(len(ref)) if log[i].tobytes() != ref[i].tobytes())
    assert first_inexact == 3699
    assert log[:first_inexact].tobytes() == ref[:first_inexact].tobytes()
    assert np.array_equal(roots[:first_inexact], z["roots"][:first_inexact])
    for field in DISCRETE:
        assert np.array_equal(log[field], ref[field]), field
    time, ref_time = log["time_q"] + log["time_r"], ref["time_q"] + ref["time_r"]
    assert np.max(np.abs(time - ref_time) / ref_time) < 1e-14
    for axis in "xyz":
        assert np.max(np.abs(log[axis] - ref[axis])) < 1e-11
    assert np.max(np.abs(roots - z["roots"])) < 1e-11


def test_square_of_the_divergence():
    """The C library's pow squares 1.0750481431014438 one unit in the last place below the correctly rounded
    square (the value CPython's ``**`` returned in the reference run)."""
    x = 1.0750481431014438
    assert x * x == 1.1557285099858625
    assert abs(1.1557285099858623 - x * x) == np.spacing(1.1557285099858623)


def test_bounds_and_walker_inputs():
    for name in ("water_n8_cell_veto", "water_n64_cell_veto", "water_n8_cell_boundaries", "water_n8_cell_bounding",
                 "water_n64_cell_bounding"):
        z, spec = load(name)
        m, layers = spec["cells_per_side"], spec["neighbor_layers"]
        upper, lower = z["bounds_upper"], z["bounds_lower"]
        near = np.zeros(m, dtype=bool)
        for o in range(-layers, layers + 1):
            near[o % m] = True
        nearby = np.array([near[c % m] and near[(c // m) % m] and near[c // (m * m)] for c in range(m ** 3)])
        assert np.all(np.isnan(upper[nearby])) and np.all(np.isnan(lower[nearby]))
        assert np.all(upper[~nearby] > 0) and np.all(upper[~nearby] <= spec["empirical_bound"])
        # the dipole estimator's lower bound is the negated upper bound, stored negated
        assert np.array_equal(upper[~nearby], lower[~nearby])
