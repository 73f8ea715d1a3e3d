"""Molecular cell-bounding and cell-veto events on the GPU through the C ABI against the reference's recorded events
and the oracle.

Bars: bounding rates and event time displacements bit for bit (a few correctly rounded products and quotients);
out-states: the thinning outcome and the new active unit equal the reference's, the event rate within 1e-12 relative
(the device's merged-image Coulomb derivative matches the reference's to 1e-12).  In the larger batches against the
oracle, events whose outcome flips when the draws move by 1e-9 relative are too close to a tie for that bar and are
counted, not compared.
"""
import math

import numpy as np
import pytest

import oracle
from tests.composite_cell_cases import bound_tables, load_cell_systems, model_of, out_arrays, time_arrays

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL = 1e-12
SYSTEMS = load_cell_systems()


@pytest.fixture(scope="module")
def composite():
    from jellyfysh_gb300 import _lib, composite as module
    _lib.load()
    return module


def _model(composite, record):
    m = model_of(record)
    return composite.CompositeModel(units=m["units"], system_length=m["system_length"], lifting=m["scheme"],
                                    alpha=m["alpha"], fourier_cutoff=m["fourier_cutoff"],
                                    position_cutoff=m["position_cutoff"], coulomb_prefactor=m["coulomb_prefactor"])


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_event_times_match_the_reference(composite, name):
    record = SYSTEMS[name]
    bounds = composite.CellBounds(*bound_tables(record))
    t = time_arrays(record)
    if record["kind"] == "cell_bounding":
        rate, time, status = composite.cell_bound_time(bounds, t["relative_cell"], t["velocity"], t["active_charge"],
                                                       t["target_charges"], record["tables"]["dipole_charge"],
                                                       t["potential_change"])
    else:
        rate, time, status = composite.cell_veto_time(bounds, t["relative_cell"], t["velocity"], t["active_charge"],
                                                      t["potential_change"])
    assert (status == 0).all()
    assert rate.tolist() == t["rate"].tolist()
    for i in range(len(time)):
        assert oracle.time_add(t["time_stamp"][i][0], t["time_stamp"][i][1], time[i]) == tuple(t["event_time"][i])


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_out_states_match_the_reference(composite, name):
    record = SYSTEMS[name]
    o = out_arrays(record)
    new_active, rates, status = composite.bounded_out_state(
        _model(composite, record), o["velocity"], o["local_positions"], o["local_charges"], o["active_index"],
        o["target_positions"], o["target_charges"], o["local_first"], o["given_rate"], o["draws"])
    assert (status == 0).all()
    assert new_active.tolist() == o["new_active"].tolist()
    assert rates[:, 0].tolist() == o["given_rate"].tolist()
    accepted = new_active >= 0
    np.testing.assert_allclose(rates[accepted, 1], o["event_rate"][accepted], rtol=REL, atol=0.0)


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_unit_draw_batches_match_the_oracle(composite, name):
    """Recorded out-states with every unit moved by up to 2% of the box and the given rate scaled by 0.5-2: new
    geometries and rates of the same kind, with unit draws, against the oracle."""
    record = SYSTEMS[name]
    model = model_of(record)
    rng = np.random.default_rng(sum(map(ord, name)))
    base = out_arrays(record)
    copies = 8
    o = {key: np.concatenate([value] * copies) for key, value in base.items()}
    length = float(record["system_length"])
    for key in ("local_positions", "target_positions"):
        o[key] = np.mod(o[key] + rng.uniform(-0.02, 0.02, o[key].shape) * length, length)
    o["draws"] = rng.random(o["draws"].shape)
    o["given_rate"] = o["given_rate"] * rng.uniform(0.5, 2.0, len(o["given_rate"]))
    new_active, rates, status = composite.bounded_out_state(
        _model(composite, record), o["velocity"], o["local_positions"], o["local_charges"], o["active_index"],
        o["target_positions"], o["target_charges"], o["local_first"], o["given_rate"], o["draws"], unit_draws=True)
    compared = 0
    for i in range(len(new_active)):
        args = (model, model["scheme"], o["velocity"][i], o["local_positions"][i], o["local_charges"][i],
                o["active_index"][i], o["target_positions"][i], o["target_charges"][i], o["local_first"][i],
                o["given_rate"][i])
        want = oracle.composite_bounded_out_state(*args, o["draws"][i], unit_draw=True)
        outcomes = {oracle.composite_bounded_out_state(*args, o["draws"][i] * f, unit_draw=True)[:2]
                    for f in (1.0 - 1e-9, 1.0 + 1e-9)}
        if len(outcomes | {want[:2]}) > 1:
            continue
        compared += 1
        assert (int(status[i]), int(new_active[i])) == want[:2], i
        assert rates[i, 0] == o["given_rate"][i]
        if want[1] >= 0:
            assert abs(rates[i, 1] - want[2]) <= REL * abs(want[2])
    assert compared >= 0.95 * len(new_active) and (new_active >= 0).any() and (new_active == -1).any()


def test_statuses_and_empty_batches(composite):
    from jellyfysh_gb300 import _lib
    nan = math.nan
    bounds = composite.CellBounds([[1.0, 2.0, 3.0], [nan, nan, nan]], [[-1.0, -2.0, -3.0], [nan, nan, nan]],
                                  [4.0, 5.0, 6.0], [7.0, 8.0, 9.0])
    x, xy = [1.0, 0.0, 0.0], [1.0, 1.0, 0.0]
    rate, time, status = composite.cell_bound_time(
        bounds, [0, 0, 1, 2, -1, 0, 0], [x, [0.0, 2.0, 0.0], x, x, x, xy, x], [1.0, -1.0, 1.0, 1.0, 1.0, 1.0, 1.0],
        [[1.0, -1.0]] * 6 + [[1.0, -0.5]], 1.0, [0.5] * 7)
    assert status.tolist() == [0, 0, _lib.STATUS_ASSERTION, _lib.STATUS_INDEX, _lib.STATUS_INDEX,
                               _lib.STATUS_ASSERTION, _lib.STATUS_ASSERTION]
    assert rate[0] == 1.0 and time[0] == 0.5
    assert rate[1] == 2.0 and time[1] == 0.125  # negative product: the lower bound times it
    # the cell veto's lower bounds are stored as magnitudes; a rate that is not positive is an assertion
    veto = composite.CellBounds([[1.0, 2.0, 3.0], [nan, nan, nan]], [[0.5, 0.25, 0.125], [nan, nan, nan]],
                                [4.0, 5.0, 6.0], [7.0, 8.0, 9.0])
    rate, time, status = composite.cell_veto_time(veto, [0, 0, 1], [x, x, x], [-0.5, 2.0, 1.0], [1.0, 1.0, 1.0])
    assert status.tolist() == [0, 0, _lib.STATUS_ASSERTION]
    assert rate[0] == 0.25 and time[0] == 1.0 / (7.0 * 0.5)
    assert rate[1] == 2.0 and time[1] == 1.0 / (4.0 * 2.0)
    with pytest.raises(ValueError):
        composite.cell_veto_time(bounds_without_walkers := composite.CellBounds([[1.0] * 3], [[1.0] * 3]), [0], [x],
                                 [1.0], [1.0])
    assert bounds_without_walkers.walker_upper is None
    empty = composite.cell_veto_time(veto, np.zeros(0), np.zeros((0, 3)), np.zeros(0), np.zeros(0))
    assert all(len(part) == 0 for part in empty)
    record = SYSTEMS["dipoles_cell_bounding"]
    o = out_arrays(record)
    _, _, status = composite.bounded_out_state(
        _model(composite, record), o["velocity"][:1], o["local_positions"][:1], o["local_charges"][:1],
        o["active_index"][:1], o["target_positions"][:1], o["target_charges"][:1], o["local_first"][:1], [-1.0],
        o["draws"][:1])
    assert status.tolist() == [_lib.STATUS_ASSERTION]


@pytest.mark.parametrize("name", ["dipoles_cell_veto", "water_cell_veto"])
def test_walker_tables_and_samples_match_the_reference(composite, name):
    from tests.composite_cell_cases import walker_draws, walkers
    record = SYSTEMS[name]
    tables = {}
    for key, w in walkers(record).items():
        table = composite.WalkerTable(w["items"], w["rates"])
        assert [list(e) for e in zip(table.first_item_host.tolist(), table.first_rate_host.tolist(),
                                     table.second_item_host.tolist())] == [list(e) for e in w["table"]]
        assert (table.total_rate, table.mean_rate) == (w["total_rate"], w["mean_rate"])
        tables[key] = table
    draws = walker_draws(record)
    for key, table in tables.items():
        mine = [row for row in draws if (row[0], row[1]) == key]
        if not mine:
            continue
        items, status = composite.walker_sample(table, [row[2] for row in mine], [row[3] for row in mine])
        assert (status == 0).all()
        assert items.tolist() == [row[4] for row in mine]


def test_walker_sampling_of_unit_draws_matches_the_oracle(composite):
    """Seeded tables of uneven rates: every entry of a 4000-sample batch of unit draws picks the oracle's item, and
    an index outside the table is an _INDEX status."""
    from jellyfysh_gb300 import _lib
    rng = np.random.default_rng(17)
    items = list(range(100, 191))
    rates = rng.exponential(1.0, len(items)) * (rng.random(len(items)) < 0.8)
    table = composite.WalkerTable(items, rates)
    status, first_item, first_rate, second_item, total, mean = oracle.walker_table(items, rates)
    assert status == 0 and (table.total_rate, table.mean_rate) == (total, mean)
    choices = rng.integers(0, len(items), 4000)
    units = rng.random(4000)
    got, st = composite.walker_sample(table, choices, units, unit_draws=True)
    assert (st == 0).all()
    want = [oracle.walker_pick(first_item, first_rate, second_item, k, 0.0 + (mean - 0.0) * u)
            for k, u in zip(choices, units)]
    assert got.tolist() == want
    _, st = composite.walker_sample(table, [len(items), -1], [0.5, 0.5], unit_draws=True)
    assert st.tolist() == [_lib.STATUS_INDEX, _lib.STATUS_INDEX]
    with pytest.raises(_lib.JfgpuError):
        composite.WalkerTable([1, 2], [1.0, -1.0])  # a negative rate fails the reference's assertion
