"""Events of two composite objects on the GPU through the C ABI against the reference's recorded events and the oracle.

Bars: the thinning outcome and the new active unit are discrete and must equal the reference's; event times and
rates are FP64 within 1e-12 relative (the merged-image Coulomb derivative on the GPU matches the reference's to
1e-12, not bit for bit, because its exponentials and error functions are the device's).  In the larger batches
against the oracle, events whose outcome flips when the draws move by 1e-9 relative are too close to a tie for
that bar and are counted, not compared.
"""
import numpy as np
import pytest

import oracle
from tests.composite_cases import load_systems, model_of, out_state_arrays, time_arrays

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL = 1e-12
SYSTEMS = load_systems()


@pytest.fixture(scope="module")
def composite():
    from jellyfysh_gb300 import _lib, composite as module
    _lib.load()
    return module


def _model(composite, record):
    m = model_of(record)
    return composite.CompositeModel(units=m["units"], system_length=m["system_length"], lifting=m["scheme"],
                                    alpha=m["alpha"], fourier_cutoff=m["fourier_cutoff"],
                                    position_cutoff=m["position_cutoff"], coulomb_prefactor=m["coulomb_prefactor"],
                                    bound_prefactor=m["bound_prefactor"])


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_event_times_match_the_reference(composite, name):
    record = SYSTEMS[name]
    t = time_arrays(record)
    displacement, status = composite.event_time(_model(composite, record), t["velocity"], t["active_position"],
                                                t["active_charge"], t["target_positions"], t["target_charges"],
                                                t["potential_changes"])
    assert (status == 0).all()
    np.testing.assert_allclose(displacement, t["expected"], rtol=REL, atol=0.0)


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_out_states_match_the_reference(composite, name):
    record = SYSTEMS[name]
    o = out_state_arrays(record)
    new_active, rates, status = composite.out_state(
        _model(composite, record), o["velocity"], o["local_positions"], o["local_charges"], o["active_index"],
        o["target_positions"], o["target_charges"], o["local_first"], o["draws"])
    assert (status == 0).all()
    assert new_active.tolist() == o["new_active"].tolist()
    np.testing.assert_allclose(rates[:, 0], o["bounding_rate"], rtol=REL, atol=0.0)
    accepted = new_active >= 0
    np.testing.assert_allclose(rates[accepted, 1], o["event_rate"][accepted], rtol=REL, atol=0.0)


def _jittered(record, rng, copies):
    """Recorded out-states with every unit moved by up to 2% of the box: new geometries of the same kind."""
    o = out_state_arrays(record)
    length = float(record["system_length"])
    out = {key: np.concatenate([value] * copies) for key, value in o.items()}
    for key in ("local_positions", "target_positions"):
        out[key] = np.mod(out[key] + rng.uniform(-0.02, 0.02, out[key].shape) * length, length)
    out["draws"] = rng.random(out["draws"].shape)
    out["local_first"] = rng.integers(0, 2, len(out["local_first"])).astype(np.int32)
    return out


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_unit_draw_batches_match_the_oracle(composite, name):
    record = SYSTEMS[name]
    model = model_of(record)
    rng = np.random.default_rng(sum(map(ord, name)))
    o = _jittered(record, rng, 8)
    new_active, rates, status = composite.out_state(
        _model(composite, record), o["velocity"], o["local_positions"], o["local_charges"], o["active_index"],
        o["target_positions"], o["target_charges"], o["local_first"], o["draws"], unit_draws=True)
    compared = near_ties = 0
    for i in range(len(new_active)):
        args = (model, model["scheme"], o["velocity"][i], o["local_positions"][i], o["local_charges"][i],
                o["active_index"][i], o["target_positions"][i], o["target_charges"][i], o["local_first"][i])
        want = oracle.composite_out_state(*args, o["draws"][i], unit_draw=True)
        outcomes = {oracle.composite_out_state(*args, o["draws"][i] * f, unit_draw=True)[:2]
                    for f in (1.0 - 1e-9, 1.0 + 1e-9)}
        if len(outcomes | {want[:2]}) > 1:
            near_ties += 1
            continue
        compared += 1
        assert (int(status[i]), int(new_active[i])) == want[:2], i
        assert abs(rates[i, 0] - want[2]) <= REL * abs(want[2])
        if want[1] >= 0:
            assert abs(rates[i, 1] - want[3]) <= REL * abs(want[3])
    assert compared >= 0.95 * len(new_active) and (new_active >= 0).any() and (new_active == -1).any()


def test_invalid_descriptions_are_argument_errors(composite):
    from jellyfysh_gb300 import _lib
    bad = composite.CompositeModel(units=9, system_length=1.0)  # more units than an object may hold
    with pytest.raises(_lib.JfgpuError):
        composite.event_time(bad, [[1.0, 0.0, 0.0]], [[0.1, 0.2, 0.3]], [1.0], np.zeros((1, 9, 3)), np.ones((1, 9)),
                             np.ones((1, 9)))
    empty = composite.CompositeModel(units=2, system_length=1.0)
    displacement, status = composite.event_time(empty, np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0),
                                                np.zeros((0, 2, 3)), np.zeros((0, 2)), np.zeros((0, 2)))
    assert len(displacement) == 0 and len(status) == 0
