"""The oracle's molecular cell-bounding and cell-veto handlers against events recorded from the reference's own runs
(dipoles with the cell-bounding potential, dipoles and water with the cell veto).

Bars: bounding rates and event times bit for bit (the handlers' arithmetic is a few products and quotients);
out-states: the thinning outcome, the new active unit and both random.uniform bounds (the given bounding rate and the
event rate of the lifting insert) bit for bit.
"""
import math

import numpy as np
import pytest

import oracle

ASSERT, ZERO_DIVISION = 2, 3  # JFO_ASSERT, JFO_ZERO_DIVISION (oracle/jf_oracle.h)
from tests.composite_cell_cases import bound_tables, load_cell_systems, model_of, out_arrays, time_arrays

SYSTEMS = load_cell_systems()


def test_every_configuration_was_recorded():
    assert set(SYSTEMS) == {"dipoles_cell_bounding", "dipoles_cell_veto", "water_cell_veto"}
    for record in SYSTEMS.values():
        outs = record["out_states"]
        assert len(record["times"]) >= 50 and len(outs) >= 30
        assert any(e["accepted"] for e in outs) and not all(e["accepted"] for e in outs)


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_event_times_match_the_reference(name):
    record = SYSTEMS[name]
    upper, lower, walker_upper, walker_lower = bound_tables(record)
    t = time_arrays(record)
    for i in range(len(t["rate"])):
        cell = t["relative_cell"][i]
        if record["kind"] == "cell_bounding":
            status, rate, time = oracle.composite_cell_bound_time(
                upper[cell], lower[cell], t["velocity"][i], t["active_charge"][i], t["target_charges"][i],
                record["tables"]["dipole_charge"], t["potential_change"][i])
        else:
            status, rate, time = oracle.composite_cell_veto_time(
                upper[cell], lower[cell], walker_upper, walker_lower, t["velocity"][i], t["active_charge"][i],
                t["potential_change"][i])
            d = int(np.nonzero(t["velocity"][i])[0][0])
            walker = walker_upper if t["active_charge"][i] > 0.0 else walker_lower
            assert walker[d] == t["walker_total"][i]
        assert status == 0
        assert rate == t["rate"][i]
        q, r = oracle.time_add(t["time_stamp"][i][0], t["time_stamp"][i][1], time)
        assert (q, r) == tuple(t["event_time"][i]), i


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_out_states_match_the_reference(name):
    record = SYSTEMS[name]
    model = model_of(record)
    o = out_arrays(record)
    for i in range(len(o["new_active"])):
        assert o["bounding_rate"][i] == o["given_rate"][i]  # the thinning draw's bound is the handler's rate
        status, new_active, rate = oracle.composite_bounded_out_state(
            model, model["scheme"], o["velocity"][i], o["local_positions"][i], o["local_charges"][i],
            o["active_index"][i], o["target_positions"][i], o["target_charges"][i], o["local_first"][i],
            o["given_rate"][i], o["draws"][i])
        assert status == 0
        assert new_active == o["new_active"][i], i
        if new_active >= 0:
            assert rate == o["event_rate"][i], i


def test_handler_assertions():
    upper, lower = [1.0, 2.0, 3.0], [-1.0, -2.0, -3.0]
    x = [1.0, 0.0, 0.0]
    ok = oracle.composite_cell_bound_time(upper, lower, x, 1.0, [1.0, -1.0], 1.0, 0.5)
    assert ok == (0, 1.0, 0.5)
    # a negative charge product takes the lower bound (a negative rate: no event)
    status, rate, time = oracle.composite_cell_bound_time(upper, lower, [0.0, 2.0, 0.0], -1.0, [1.0, -1.0], 1.0, 0.5)
    assert status == 0 and rate == 2.0 and time == 0.125
    status, rate, time = oracle.composite_cell_bound_time(upper, [1.0, 1.0, 1.0], x, -1.0, [1.0, -1.0], 1.0, 0.5)
    assert status == 0 and rate == -1.0 and math.isinf(time)
    nan = [math.nan] * 3
    assert oracle.composite_cell_bound_time(nan, nan, x, 1.0, [1.0, -1.0], 1.0, 0.5)[0] == ASSERT
    assert oracle.composite_cell_bound_time(upper, lower, x, 1.0, [1.0, -0.5], 1.0, 0.5)[0] == ASSERT
    assert oracle.composite_cell_bound_time(upper, lower, [1.0, 1.0, 0.0], 1.0, [1.0, -1.0], 1.0, 0.5)[0] == \
        ASSERT
    assert oracle.composite_cell_bound_time(upper, lower, x, 1.0, [1.0, -1.0], 0.0, 0.5)[0] == ZERO_DIVISION
    # the cell veto: a charge of either sign takes its own bounds (the lower ones stored as magnitudes) and Walker
    # total; a rate that is not positive is an assertion
    magnitudes = [0.5, 0.25, 0.125]
    status, rate, time = oracle.composite_cell_veto_time(upper, magnitudes, [4.0, 5.0, 6.0], [7.0, 8.0, 9.0], x,
                                                         -0.5, 1.0)
    assert status == 0 and rate == 0.25 and time == 1.0 / (7.0 * 0.5)
    assert oracle.composite_cell_veto_time(upper, [0.0] * 3, [1.0] * 3, [1.0] * 3, x, -1.0, 1.0)[0] == ASSERT
    # a negative given bounding rate fails the handlers' assertion
    record = SYSTEMS["dipoles_cell_bounding"]
    model = model_of(record)
    o = out_arrays(record)
    status = oracle.composite_bounded_out_state(
        model, model["scheme"], o["velocity"][0], o["local_positions"][0], o["local_charges"][0],
        o["active_index"][0], o["target_positions"][0], o["target_charges"][0], o["local_first"][0], -1.0,
        o["draws"][0])[0]
    assert status == ASSERT


@pytest.mark.parametrize("name", ["dipoles_cell_veto", "water_cell_veto"])
def test_walker_tables_and_samples_match_the_reference(name):
    """The cell veto's alias tables (walker.py:53-103) rebuilt from the handler's items equal the reference's entry
    for entry, with its total and mean rate; every recorded sample_cell call picks the recorded relative cell."""
    from tests.composite_cell_cases import walker_draws, walkers
    record = SYSTEMS[name]
    tables = walkers(record)
    for key, w in tables.items():
        status, first_item, first_rate, second_item, total, mean = oracle.walker_table(w["items"], w["rates"])
        assert status == 0
        assert [list(entry) for entry in zip(first_item, first_rate, second_item)] == [list(e) for e in w["table"]]
        assert (total, mean) == (w["total_rate"], w["mean_rate"])
    for which, d, choice, uniform, cell in walker_draws(record):
        table = tables[(which, d)]["table"]
        picked = oracle.walker_pick([e[0] for e in table], [e[1] for e in table], [e[2] for e in table], choice,
                                    uniform)
        assert picked == cell
