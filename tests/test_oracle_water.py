"""The oracle's water event loop against trajectories of the reference's own event loop (bit-exact)."""
import numpy as np
import pytest

import oracle
from tests.water_cases import FIELDS, load_water, water_names


@pytest.mark.parametrize("name", water_names())
def test_oracle_reproduces_the_reference_water_trajectory(name):
    spec, initial, charges, events, final = load_water(name)
    water = oracle.Water(oracle.make_water_system(spec, spec["rng_key"]), initial, charges)
    log = water.run(len(events))
    assert len(log) == len(events)
    for field in FIELDS + ("time_q", "time_r", "x", "y", "z"):
        assert (log[field] == events[field]).all(), field
    assert (water.positions() == final).all()


def test_water_trajectories_cover_every_event_kind():
    kinds = set()
    for name in water_names():
        events = load_water(name)[3]
        kinds |= set(zip(events["kind"].tolist(), events["accepted"].tolist()))
    assert {(oracle.EV_COMPOSITE, 0), (oracle.EV_COMPOSITE, 1), (oracle.EV_BOND, 1), (oracle.EV_PAIR, 1),
            (oracle.EV_END_OF_CHAIN, 1)} <= kinds
    assert "water_n64" in water_names()  # the 64-molecule box of the batched water workload


def test_water_lattice_geometry():
    from jellyfysh_gb300 import systems
    positions, charges = systems.water_lattice(4, 12.42, 1.0, 1.633, np.random.default_rng(5))
    assert positions.shape == (192, 3) and (positions >= 0).all() and (positions < 12.42).all()
    assert charges.sum() == pytest.approx(0.0, abs=1e-12)
    s = positions.reshape(64, 3, 3)
    wrap = lambda v: (v + 6.21) % 12.42 - 6.21
    assert np.allclose(np.linalg.norm(wrap(s[:, 0] - s[:, 1]), axis=1), 1.0)
    assert np.allclose(np.linalg.norm(wrap(s[:, 2] - s[:, 1]), axis=1), 1.0)
    assert np.allclose(np.linalg.norm(wrap(s[:, 2] - s[:, 0]), axis=1), 1.633)


def test_water_model_matches_the_header_layouts():
    import ctypes
    from jellyfysh_gb300 import _lib, water
    assert ctypes.sizeof(_lib.WaterDesc) == 144
    assert water.STATE_DTYPE.itemsize == 120  # JfgpuWaterState: 4 doubles, 6 int32, 8 int64
    model = water.WaterModel.from_spec({"molecules_per_side": 2, "system_length": 6.21, "lifting": "ratio",
                                        "unused": 1})
    assert model.molecules == 8 and model.system_length == 6.21
    desc = model.desc(seed=7)
    assert (desc.molecules, desc.lifting, desc.seed, desc.initial_active) == (8, _lib.LIFTING_RATIO, 7, 1)
    assert desc.mode == _lib.MODE_MIXED and water.WaterModel(mode="exact").desc(0).mode == _lib.MODE_EXACT
    assert desc.oh_prefactor == 529.5 and desc.hh_prefactor == 342.0
    assert model.charges().tolist()[:3] == [0.41, -0.82, 0.41]


def test_lattice_positions_are_seeded_per_chain():
    from jellyfysh_gb300 import water
    model = water.WaterModel(molecules=8, system_length=6.21)
    a = water.lattice_positions(model, 3, seed=5)
    b = water.lattice_positions(model, 2, seed=5, rng_offset=1)
    assert a.shape == (3, 24, 3) and np.array_equal(a[1:], b)
    with pytest.raises(ValueError):
        water.lattice_positions(water.WaterModel(molecules=10), 1, seed=0)
