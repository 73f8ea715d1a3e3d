"""The oracle's event loop against event-by-event trajectories of the reference (CPU only).

The fixtures were recorded from the reference's own ``SingleProcessMediator.run`` driven with keyed random
numbers (``golden/make_reference_trajectories.py``); the oracle must reproduce every event (winner kind, target,
lifting outcome, event time, committed position) and the final configuration bit for bit.
"""
import numpy as np
import pytest

import oracle
from tests.trajectory_cases import load_trajectory, oracle_system, trajectory_names


@pytest.mark.parametrize("name", trajectory_names())
def test_oracle_reproduces_reference_trajectory(name):
    spec, initial, charges, events, final = load_trajectory(name)
    chain = oracle.Chain(oracle_system(spec), initial, charges)
    log = chain.run(len(events))
    assert len(log) == len(events)
    for field in oracle.EVENT_DTYPE.names:
        mismatch = np.nonzero(log[field] != events[field])[0]
        assert mismatch.size == 0, (field, int(mismatch[0]), log[mismatch[0]], events[mismatch[0]])
    assert np.array_equal(chain.positions(), final)


def test_fixtures_cover_every_event_kind():
    seen = set()
    for name in trajectory_names():
        seen |= set(np.unique(load_trajectory(name)[3]["kind"]).tolist())
    for kind in (oracle.EV_PAIR, oracle.EV_BOUNDED, oracle.EV_HARDCORE, oracle.EV_CELL_BOUNDING, oracle.EV_CELL_VETO,
                 oracle.EV_BOUNDARY, oracle.EV_END_OF_CHAIN):
        assert kind in seen


def test_stop_time_slices_the_active_unit():
    spec, initial, charges, events, final = load_trajectory("hard_spheres_n64")
    chain = oracle.Chain(oracle_system(spec), initial, charges)
    t_stop = float(events["time_q"][99] + events["time_r"][99]) + 1e-9
    done = chain.run(10_000, stop_time=t_stop, record=False)
    assert done == 100
    state = chain.state()
    assert state["time_q"] + state["time_r"] == pytest.approx(t_stop, abs=1e-15)
