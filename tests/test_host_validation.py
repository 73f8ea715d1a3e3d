"""Corrupted inputs stop on the host, before the device sees them: positions that are not finite or lie outside the
box, charges that are not finite (the batches raise ValueError before loading the library, so this runs on CPU)."""
import math

import numpy as np
import pytest

from jellyfysh_gb300 import ChainBatch, ChainSpec, water


@pytest.mark.parametrize("bad", [math.nan, math.inf, -1e-12, 1.0])
def test_chain_positions_outside_the_box_are_refused(bad):
    spec = ChainSpec(n=2, system_length=1.0, cells_per_side=3, hs_radius=0.1, chain_time=0.3)
    positions = np.array([[0.1, 0.2, 0.3], [0.5, 0.6, 0.7]])
    positions[1, 2] = bad
    with pytest.raises(ValueError, match="must be finite|must lie in"):
        ChainBatch([spec], [positions])


def test_chain_charges_must_be_finite():
    spec = ChainSpec(n=2, system_length=1.0, cells_per_side=3, potential="coulomb", chain_time=0.3)
    with pytest.raises(ValueError, match="must be finite|must lie in"):
        ChainBatch([spec], [np.array([[0.1, 0.2, 0.3], [0.5, 0.6, 0.7]])], charges=[np.array([1.0, math.nan])])


@pytest.mark.parametrize("bad", [math.nan, -0.5, 12.42])
def test_water_positions_outside_the_box_are_refused(bad):
    model = water.WaterModel()
    positions = water.lattice_positions(model, 1, 3)
    positions[0, 5, 1] = bad
    with pytest.raises(ValueError, match="must be finite|must lie in"):
        water.WaterBatch(model, positions)
    with pytest.raises(ValueError, match="must be finite|must lie in"):
        water.WaterBatch(model, water.lattice_positions(model, 1, 3), charges=np.full(192, math.inf))
