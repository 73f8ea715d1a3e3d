"""Events of two composite objects on the CPU: the oracle against the reference's recorded events (bit-exact), and
the host-side description of the GPU entry points (no compute)."""
import ctypes

import numpy as np
import pytest

import oracle
from jellyfysh_gb300 import _lib
from jellyfysh_gb300.composite import CompositeModel
from tests.composite_cases import load_systems, model_of, out_state_arrays, time_arrays

SYSTEMS = load_systems()


def test_fixture_covers_dipoles_water_and_every_scheme():
    schemes = {(model_of(r)["units"], model_of(r)["scheme"]) for r in SYSTEMS.values()}
    assert schemes == {(2, "inside_first"), (2, "outside_first"), (2, "ratio"), (3, "inside_first")}
    for record in SYSTEMS.values():
        arrays = out_state_arrays(record)
        assert (arrays["new_active"] == -1).sum() > 0 and (arrays["new_active"] >= 0).sum() > 0
        # both orders of the derivative table, and lifting to local as well as target units
        assert set(arrays["local_first"]) == {0, 1}
        k = model_of(record)["units"]
        assert (arrays["new_active"][arrays["new_active"] >= 0] < k).any()
        assert (arrays["new_active"] >= k).any()


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_oracle_event_times_equal_the_reference(name):
    model = model_of(SYSTEMS[name])
    t = time_arrays(SYSTEMS[name])
    for i in range(len(t["expected"])):
        status, displacement = oracle.composite_event_time(
            model, t["velocity"][i], t["active_position"][i], t["active_charge"][i], t["target_positions"][i],
            t["target_charges"][i], t["potential_changes"][i])
        assert status == 0 and displacement == t["expected"][i]


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_oracle_out_states_equal_the_reference(name):
    model = model_of(SYSTEMS[name])
    o = out_state_arrays(SYSTEMS[name])
    for i in range(len(o["new_active"])):
        status, new_active, bounding, rate = oracle.composite_out_state(
            model, model["scheme"], o["velocity"][i], o["local_positions"][i], o["local_charges"][i],
            o["active_index"][i], o["target_positions"][i], o["target_charges"][i], o["local_first"][i],
            o["draws"][i])
        assert status == 0
        assert new_active == o["new_active"][i]
        assert bounding == o["bounding_rate"][i]  # the reference's random.uniform bound, bit for bit
        if new_active >= 0:
            assert rate == o["event_rate"][i]


def test_composite_description_matches_the_header_layout():
    assert ctypes.sizeof(_lib.CompositeDesc) == 48
    desc = CompositeModel(units=3, system_length=10.0, lifting="ratio", coulomb_prefactor=332.0,
                          bound_prefactor=531.2).desc()
    assert (desc.units, desc.lifting, desc.fourier_cutoff, desc.position_cutoff) == (3, _lib.LIFTING_RATIO, 6, 2)
    assert (desc.alpha, desc.coulomb_prefactor, desc.bound_prefactor, desc.system_length) == (3.45, 332.0, 531.2,
                                                                                              10.0)
