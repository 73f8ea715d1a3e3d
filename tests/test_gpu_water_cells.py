"""Batched water with molecular cells on the GPU through the C ABI against the reference's trajectories and the
oracle.

The reference trajectories (``golden/water_*cell*.npz``, see ``tests/test_water_cells_oracle.py``) run the
reference's water cell-veto configuration: root units in cells, the Coulomb factor with the nearby and surplus
molecules, the molecular cell veto and the cell-boundary events across which the bond and Lennard-Jones candidates
persist.  Bars as for the all-pairs water: every discrete field exactly, event times to 1e-12 relative, committed
leaf and root positions to 1e-12 of the box.  The mixed mode (FP32 screen of the Coulomb candidates and of the
thinning) equals the exact mode bit for bit.
"""
import numpy as np
import pytest

import oracle
from tests.water_cases import FIELDS, load_water_cells, water_cell_names

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL = 1e-12


@pytest.fixture(scope="module")
def water():
    from jellyfysh_gb300 import _lib, water as module
    _lib.load()
    return module


def wrapped(diff, length):
    diff = np.abs(diff)
    return np.minimum(diff, length - diff)


def compare_logs(log, events, length, roots=None, ref_roots=None):
    assert len(log) == len(events)
    for field in FIELDS:
        bad = np.nonzero(log[field] != events[field])[0]
        assert bad.size == 0, (field, int(bad[0]), log[bad[0]], events[bad[0]])
    t_gpu = log["time_q"] + log["time_r"]
    t_ref = events["time_q"] + events["time_r"]
    assert np.all(np.abs(t_gpu - t_ref) <= REL * np.maximum(np.abs(t_ref), 1.0))
    for axis in ("x", "y", "z"):
        assert np.all(wrapped(log[axis] - events[axis], length) <= REL * length), axis
    if roots is not None:
        assert np.all(wrapped(roots - ref_roots, length) <= REL * length)


def cells_of(water, spec, data):
    return water.WaterCells(spec["cells_per_side"], spec["neighbor_layers"], data["bounds_upper"],
                            data["bounds_lower"], far=spec.get("far", "cell_veto"),
                            dipole_charge=spec["dipole_charge"])


def oracle_chain(spec, data, positions, roots, key, charges):
    system = oracle.make_water_system(spec, key)
    return oracle.Water(system, positions, charges, cells=(spec["cells_per_side"], spec["neighbor_layers"], roots,
                                                           data["bounds_upper"], data["bounds_lower"], True,
                                                           spec.get("far", "cell_veto"), spec["dipole_charge"]))


@pytest.mark.parametrize("mode", ["exact", "mixed"])
@pytest.mark.parametrize("name", water_cell_names())
def test_gpu_water_cells_reproduce_the_reference_trajectory(water, name, mode):
    spec, data = load_water_cells(name)
    model = water.WaterModel.from_spec(dict(spec, mode=mode))
    events = data["events"]
    batch = water.WaterBatch(model, data["initial"][None], seed=spec["seed"], charges=data["charges"],
                             cells=cells_of(water, spec, data), roots=data["initial_roots"][None])
    log, roots = batch.run(len(events), record=True, record_roots=True)
    batch.check_status()
    compare_logs(log[0], events, model.system_length, roots[0], data["roots"])
    assert np.all(wrapped(batch.positions()[0] - data["final"], model.system_length) <= REL * model.system_length)
    assert np.all(wrapped(batch.roots()[0] - data["final_roots"], model.system_length) <= REL * model.system_length)
    cell_state = batch.cell_states()[0]
    assert cell_state["boundary_events"] == np.sum(events["kind"] == oracle.EV_BOUNDARY)
    far = (events["kind"] == oracle.EV_CELL_VETO) | (events["kind"] == oracle.EV_CELL_BOUNDING)
    assert cell_state["veto_events"] == np.sum(far)
    assert cell_state["veto_targets"] == np.sum(far & (events["target"] >= 0))
    state = batch.states()[0]
    assert state["events"] == len(events)
    assert state["bond_events"] == np.sum(events["kind"] == oracle.EV_BOND)
    assert state["eoc_events"] == np.sum(events["kind"] == oracle.EV_END_OF_CHAIN)


def test_batched_chains_with_cells_match_the_oracle(water):
    """24 chains of the 64-molecule box (8^3 cells, two neighbour layers) from lattice starts of their own against
    the oracle, and the mixed mode equal to the exact mode bit for bit."""
    spec, data = load_water_cells("water_n64_cell_veto")
    chains, events, seed = 24, 600, 4321
    runs = {}
    for mode in ("exact", "mixed"):
        model = water.WaterModel.from_spec(dict(spec, mode=mode))
        positions = water.lattice_positions(model, chains, seed)
        batch = water.WaterBatch(model, positions, seed=seed, cells=cells_of(water, spec, data))
        log, roots = batch.run(events, record=True, record_roots=True)
        batch.check_status()
        runs[mode] = (log, roots, batch.positions(), batch.roots(), batch.states(), batch.cell_states(), positions,
                      model)
    log, roots, _, _, exact_states, cell_states, positions, model = runs["exact"]
    for field in log.dtype.names:
        assert np.array_equal(log[field], runs["mixed"][0][field]), field
    for k in (1, 2, 3):
        assert np.array_equal(runs["exact"][k], runs["mixed"][k])
    mixed_states = runs["mixed"][4]
    assert mixed_states["refined_items"].sum() < 0.5 * exact_states["refined_items"].sum()
    from jellyfysh_gb300 import systems
    for c in (0, 11, 23):
        roots0 = systems.water_roots(positions[c], model.system_length)
        chain = oracle_chain(spec, data, positions[c], roots0, oracle.chain_key(seed, c), model.charges())
        expected, expected_roots = chain.run(events, roots=True)
        compare_logs(log[c], expected, model.system_length, roots[c], expected_roots)
    kinds = np.bincount(log["kind"].reshape(-1), minlength=10)
    assert kinds[oracle.EV_CELL_VETO] > 0 and kinds[oracle.EV_COMPOSITE] > 0 and kinds[oracle.EV_BOND] > 0
    assert cell_states["veto_targets"].sum() > 0


def test_pieces_checkpoint_and_restore_continue_bit_for_bit(water, tmp_path):
    """Calls of any length and a checkpoint in the middle continue the chains exactly, the persistent bond and
    Lennard-Jones candidates included (the boundary-heavy geometry of water_n8_cell_boundaries)."""
    spec, data = load_water_cells("water_n8_cell_boundaries")
    model = water.WaterModel.from_spec(spec)
    positions = water.lattice_positions(model, 8, 17)
    cells = cells_of(water, spec, data)
    straight = water.WaterBatch(model, positions, seed=17, cells=cells)
    whole = straight.run(1500, record=True)
    parts = water.WaterBatch(model, positions, seed=17, cells=cells, warps_per_block=2)
    first = np.concatenate([parts.run(n, record=True) for n in (1, 299, 400)], axis=1)
    path = str(tmp_path / "water_cells.npz")
    parts.checkpoint(path)
    parts.close()
    resumed = water.WaterBatch.restore(path)
    second = resumed.run(800, record=True)
    pieces = np.concatenate([first, second], axis=1)
    for field in whole.dtype.names:
        assert np.array_equal(whole[field], pieces[field]), field
    assert np.array_equal(straight.positions(), resumed.positions())
    assert np.array_equal(straight.roots(), resumed.roots())
    assert np.array_equal(straight.cell_states(), resumed.cell_states())
    assert straight.cell_states()["boundary_events"].sum() > 20


def test_device_dipole_estimator_agrees_with_the_reference_tables(water):
    """The molecular cell veto's bound tables from the device dipole estimator (other random dipoles than the
    reference's, the same estimator) against the reference's tables of the 64-molecule box: the same far cells, and
    the maxima over 1000 random dipoles alike in distribution (the maximum of a heavy-tailed sample: the median ratio
    within 5 %, nine in ten within 25 %, all within a factor two)."""
    spec, data = load_water_cells("water_n64_cell_veto")
    model = water.WaterModel.from_spec(spec)
    cells = water.dipole_cell_veto_bounds(model, spec["cells_per_side"], spec["neighbor_layers"],
                                          spec["dipole_separation"], spec["dipole_charge"],
                                          spec["estimator_prefactor"], spec["number_trials"],
                                          spec["empirical_bound"], seed=3)
    reference = data["bounds_upper"]
    far = ~np.isnan(reference[:, 0])
    assert np.array_equal(np.isnan(cells.bounds_upper), np.isnan(reference))
    assert np.array_equal(cells.bounds_upper[far], cells.bounds_lower[far])
    ratio = cells.bounds_upper[far] / reference[far]
    assert abs(np.median(ratio) - 1.0) < 0.05
    assert np.mean((ratio > 0.8) & (ratio < 1.25)) > 0.9
    assert np.all((ratio > 0.5) & (ratio < 2.0)), (ratio.min(), ratio.max())


def test_drop_in_plan_with_molecular_cells_runs_to_its_end_of_run_time(water):
    """The drop-in mediator's water plan with molecular cells (as ``plugin.plan`` reads it from the reference's water
    cell-veto configuration): the bound tables from the device dipole estimator, every chain stopped at the end-of-run
    time, the same chains as a batch built directly; with keep_pairs off the pair candidates do not outlive a cell
    boundary, as the oracle's loop with that setting."""
    from jellyfysh_gb300.plugin.plan import WaterPlan, run_plan
    spec, data = load_water_cells("water_n8_cell_boundaries")
    model = water.WaterModel.from_spec(spec)
    cell_veto = dict(cells_per_side=spec["cells_per_side"], neighbor_layers=spec["neighbor_layers"],
                     dipole_separation=spec["dipole_separation"], dipole_charge=spec["dipole_charge"],
                     prefactor=spec["estimator_prefactor"], number_trials=200, empirical_bound=spec["empirical_bound"],
                     keep_pairs=True)
    plan = WaterPlan(model=model, positions=data["initial"], charges=data["charges"], end_of_run_time=40.0, chains=3,
                     seed=spec["seed"], events_per_launch=300, roots=data["initial_roots"], cell_veto=cell_veto)
    batch = run_plan(plan)
    states = batch.states()
    assert (states["stopped"] == 1).all() and (states["time_q"] + states["time_r"] == 40.0).all()
    assert batch.cell_states()["boundary_events"].sum() > 0
    cells = water.dipole_cell_veto_bounds(model, seed=spec["seed"], **cell_veto)
    direct = water.WaterBatch(model, np.repeat(data["initial"][None], 3, axis=0), seed=spec["seed"],
                              charges=data["charges"], cells=cells, roots=np.repeat(data["initial_roots"][None], 3, 0))
    direct.run(int(states["events"][0]) + 10, stop_time=40.0)
    assert np.array_equal(direct.positions(), batch.positions())
    assert np.array_equal(direct.roots(), batch.roots())
    # keep_pairs off against the oracle's loop with the same setting
    trashing = water.WaterCells(spec["cells_per_side"], spec["neighbor_layers"], data["bounds_upper"],
                                data["bounds_lower"], keep_pairs=False)
    events = 2000
    gpu = water.WaterBatch(model, data["initial"][None], seed=spec["seed"], charges=data["charges"], cells=trashing,
                           roots=data["initial_roots"][None])
    log, roots = gpu.run(events, record=True, record_roots=True)
    gpu.check_status()
    chain = oracle.Water(oracle.make_water_system(spec, spec["rng_key"]), data["initial"], data["charges"],
                         cells=(spec["cells_per_side"], spec["neighbor_layers"], data["initial_roots"],
                                data["bounds_upper"], data["bounds_lower"], False))
    expected, expected_roots = chain.run(events, roots=True)
    compare_logs(log[0], expected, model.system_length, roots[0], expected_roots)
    assert np.sum(expected["kind"] == oracle.EV_BOUNDARY) > 10


def test_batched_chains_with_cell_bounding_match_the_oracle(water):
    """16 chains of the 64-molecule box with the molecular cell-bounding far field (6^3 cells, one layer) from lattice
    starts of their own against the oracle, and the mixed mode (the far factors screened in FP32) equal to the exact
    mode bit for bit."""
    spec, data = load_water_cells("water_n64_cell_bounding")
    chains, events, seed = 16, 500, 2468
    runs = {}
    for mode in ("exact", "mixed"):
        model = water.WaterModel.from_spec(dict(spec, mode=mode))
        positions = water.lattice_positions(model, chains, seed)
        batch = water.WaterBatch(model, positions, seed=seed, cells=cells_of(water, spec, data))
        log, roots = batch.run(events, record=True, record_roots=True)
        batch.check_status()
        runs[mode] = (log, roots, batch.positions(), batch.states(), positions, model)
    log, roots, final, states, positions, model = runs["exact"]
    for field in log.dtype.names:
        assert np.array_equal(log[field], runs["mixed"][0][field]), field
    assert np.array_equal(roots, runs["mixed"][1]) and np.array_equal(final, runs["mixed"][2])
    assert runs["mixed"][3]["refined_items"].sum() < 0.5 * states["refined_items"].sum()
    from jellyfysh_gb300 import systems
    for c in (0, 9, 15):
        roots0 = systems.water_roots(positions[c], model.system_length)
        chain = oracle_chain(spec, data, positions[c], roots0, oracle.chain_key(seed, c), model.charges())
        expected, expected_roots = chain.run(events, roots=True)
        compare_logs(log[c], expected, model.system_length, roots[c], expected_roots)
    assert np.sum(log["kind"] == oracle.EV_CELL_BOUNDING) > 0
