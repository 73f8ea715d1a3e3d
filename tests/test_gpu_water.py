"""Batched water chains on the GPU through the C ABI against the reference's water trajectories and the oracle.

Bars, as for the atomic trajectories: kind, moved unit, target, new active unit, direction and thinning outcome of
every event exactly; event times to 1e-12 relative and committed positions to 1e-12 of the box (the device's
merged-image Coulomb derivative, exponentials and powers agree with the reference's to about an ulp, not bit for
bit).
"""
import numpy as np
import pytest

import oracle
from tests.water_cases import FIELDS, load_water, water_names

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL = 1e-12


@pytest.fixture(scope="module")
def water():
    from jellyfysh_gb300 import _lib, water as module
    _lib.load()
    return module


def compare_logs(log, events, length):
    assert len(log) == len(events)
    for field in FIELDS:
        bad = np.nonzero(log[field] != events[field])[0]
        assert bad.size == 0, (field, int(bad[0]), log[bad[0]], events[bad[0]])
    t_gpu = log["time_q"] + log["time_r"]
    t_ref = events["time_q"] + events["time_r"]
    assert np.all(np.abs(t_gpu - t_ref) <= REL * np.maximum(np.abs(t_ref), 1.0))
    for axis in ("x", "y", "z"):
        diff = np.abs(log[axis] - events[axis])
        diff = np.minimum(diff, length - diff)
        assert np.all(diff <= REL * length), (axis, float(diff.max()))


@pytest.mark.parametrize("name", water_names())
def test_gpu_water_reproduces_the_reference_trajectory(water, name):
    spec, initial, charges, events, final = load_water(name)
    model = water.WaterModel.from_spec(spec)
    batch = water.WaterBatch(model, initial[None], seed=spec["seed"], charges=charges)
    log = batch.run(len(events), record=True)[0]
    batch.check_status()
    compare_logs(log, events, model.system_length)
    diff = np.abs(batch.positions()[0] - final)
    assert np.all(np.minimum(diff, model.system_length - diff) <= REL * model.system_length)
    state = batch.states()[0]
    assert state["events"] == len(events)
    assert state["composite_events"] == np.sum(events["kind"] == oracle.EV_COMPOSITE)
    assert state["composite_accepted"] == np.sum((events["kind"] == oracle.EV_COMPOSITE) & (events["accepted"] == 1))
    assert state["bond_events"] == np.sum(events["kind"] == oracle.EV_BOND)
    assert state["lj_events"] == np.sum(events["kind"] == oracle.EV_PAIR)
    assert state["eoc_events"] == np.sum(events["kind"] == oracle.EV_END_OF_CHAIN)


def test_gpu_water_in_pieces_equals_one_run(water):
    spec, initial, charges, events, final = load_water("water_n8")
    model = water.WaterModel.from_spec(spec)
    whole = water.WaterBatch(model, initial[None], seed=spec["seed"], charges=charges)
    one = whole.run(600, record=True)[0]
    parts = water.WaterBatch(model, initial[None], seed=spec["seed"], charges=charges, warps_per_block=2)
    pieces = np.concatenate([parts.run(n, record=True)[0] for n in (1, 99, 250, 250)])
    for field in one.dtype.names:
        assert np.array_equal(one[field], pieces[field]), field
    assert np.array_equal(whole.positions(), parts.positions())


def test_batched_water_chains_match_the_oracle(water):
    """64 chains of the 64-molecule box (lattice starts of their own, keys of their own) against the oracle."""
    model = water.WaterModel()
    chains, events, seed = 64, 300, 1234
    positions = water.lattice_positions(model, chains, seed)
    batch = water.WaterBatch(model, positions, seed=seed)
    log = batch.run(events, record=True)
    batch.check_status()
    spec = dict(vars(model))
    for c in (0, 1, 31, 63):
        reference = oracle.Water(oracle.make_water_system(spec, oracle.chain_key(seed, c)), positions[c],
                                 model.charges())
        compare_logs(log[c], reference.run(events), model.system_length)
    kinds = np.bincount(log["kind"].reshape(-1), minlength=10)
    assert kinds[oracle.EV_COMPOSITE] > 0 and kinds[oracle.EV_BOND] > 0


def test_mixed_mode_equals_exact_mode(water):
    """The FP32-screened rejections of the mixed mode leave every event, time and position as in the exact mode."""
    chains, events, seed = 96, 200, 77
    runs = {}
    for mode in ("exact", "mixed"):
        model = water.WaterModel(mode=mode)
        batch = water.WaterBatch(model, water.lattice_positions(model, chains, seed), seed=seed)
        runs[mode] = (batch.run(events, record=True), batch.positions(), batch.states())
        batch.check_status()
    for field in runs["exact"][0].dtype.names:
        assert np.array_equal(runs["exact"][0][field], runs["mixed"][0][field]), field
    assert np.array_equal(runs["exact"][1], runs["mixed"][1])
    exact, mixed = runs["exact"][2], runs["mixed"][2]
    assert (exact["thinning_exact"] == exact["composite_events"]).all()
    # most rejections are decided by the FP32 sums, most candidates by the FP32 screen
    assert mixed["thinning_exact"].sum() < 0.5 * mixed["composite_events"].sum()
    assert mixed["refined_items"].sum() < 0.2 * exact["refined_items"].sum()


def test_water_replicas_of_the_batched_workload_run_clean(water):
    """512 replicas of 64 molecules: every chain advances without a status, positions stay in the box."""
    model = water.WaterModel()
    positions = water.lattice_positions(model, 512, 99)
    batch = water.WaterBatch(model, positions, seed=99)
    batch.run(100)
    batch.check_status()
    states = batch.states()
    assert (states["events"] == 100).all()
    final = batch.positions()
    assert np.isfinite(final).all() and (final >= 0).all() and (final < model.system_length).all()


def test_stop_time_time_slices_the_active_unit(water):
    """A run with a stop time ends like the reference's end of run: the events before it, then the active unit
    time-sliced to the stop time; the drop-in plan runs every chain to its end-of-run time."""
    spec, initial, charges, events, final = load_water("water_n8")
    model = water.WaterModel.from_spec(spec)
    k = 150
    t_k = events["time_q"][k] + events["time_r"][k]
    t_next = events["time_q"][k + 1] + events["time_r"][k + 1]
    stop = 0.5 * (t_k + t_next)
    before = water.WaterBatch(model, initial[None], seed=spec["seed"], charges=charges)
    before.run(k + 1)
    stopped = water.WaterBatch(model, initial[None], seed=spec["seed"], charges=charges)
    stopped.run(1000, stop_time=stop)
    stopped.check_status()
    state = stopped.states()[0]
    assert state["stopped"] == 1 and state["events"] == k + 1
    assert (state["time_q"], state["time_r"]) == divmod(stop, 1.0)
    expected = before.positions()[0].copy()
    active, direction = int(state["active"]), int(state["direction"])
    dt = (divmod(stop, 1.0)[0] - events["time_q"][k]) + divmod(stop, 1.0)[1] - events["time_r"][k]
    expected[active, direction] = (expected[active, direction] + dt) % model.system_length
    assert np.allclose(stopped.positions()[0], expected, rtol=0, atol=REL * model.system_length)
    # a second call at the same stop time does nothing
    stopped.run(10, stop_time=stop)
    assert stopped.states()[0]["events"] == k + 1

    from jellyfysh_gb300.plugin.plan import WaterPlan, run_plan
    plan = WaterPlan(model=model, positions=initial, charges=charges, end_of_run_time=stop, chains=3, seed=spec["seed"],
                     events_per_launch=64)
    batch = run_plan(plan)
    states = batch.states()
    assert (states["stopped"] == 1).all() and (states["time_q"] + states["time_r"] == stop).all()
    assert states["events"][0] == k + 1  # chain 0 draws the keys of the recorded trajectory


def test_checkpoint_and_restore_continue_bit_for_bit(water, tmp_path):
    model = water.WaterModel()
    positions = water.lattice_positions(model, 16, 5)
    straight = water.WaterBatch(model, positions, seed=5)
    straight.run(300)
    reference = straight.run(200, record=True)
    interrupted = water.WaterBatch(model, positions, seed=5)
    interrupted.run(300)
    path = str(tmp_path / "water.npz")
    interrupted.checkpoint(path)
    interrupted.close()
    resumed = water.WaterBatch.restore(path)
    continued = resumed.run(200, record=True)
    for field in reference.dtype.names:
        assert np.array_equal(reference[field], continued[field]), field
    assert np.array_equal(straight.positions(), resumed.positions())
    assert np.array_equal(straight.states(), resumed.states())


@pytest.mark.parametrize("lifting", ["outside_first", "ratio"])
def test_other_lifting_schemes_match_the_oracle(water, lifting):
    """The water engine with the outside-first and ratio schemes against the oracle, mixed and exact modes."""
    chains, events, seed = 24, 300, 61
    for mode in ("mixed", "exact"):
        model = water.WaterModel(lifting=lifting, mode=mode)
        positions = water.lattice_positions(model, chains, seed)
        batch = water.WaterBatch(model, positions, seed=seed)
        log = batch.run(events, record=True)
        batch.check_status()
        spec = dict(vars(model))
        for c in (0, 7, 23):
            reference = oracle.Water(oracle.make_water_system(spec, oracle.chain_key(seed, c)), positions[c],
                                     model.charges())
            compare_logs(log[c], reference.run(events), model.system_length)
        assert (log["kind"] == oracle.EV_COMPOSITE).any() and ((log["kind"] == oracle.EV_COMPOSITE) &
                                                              (log["accepted"] == 1)).any()


def test_invalid_descriptions_and_launch_shapes_are_errors(water):
    """The C ABI refuses a model it cannot run (fewer than two molecules, an initial active unit outside the system)
    and more than eight warps a chain, with an argument error; a box that is not positive stops on the host."""
    from jellyfysh_gb300 import _lib
    for bad in (water.WaterModel(molecules=1), water.WaterModel(initial_active=3 * 64)):
        with pytest.raises(_lib.JfgpuError):
            water.WaterBatch(bad, np.zeros((1, 3 * bad.molecules, 3)), seed=0)
    with pytest.raises(ValueError, match="must lie in"):  # no position lies in a box that is not positive
        water.WaterBatch(water.WaterModel(system_length=-1.0), np.zeros((1, 192, 3)), seed=0)
    model = water.WaterModel(molecules=8, system_length=6.21)
    batch = water.WaterBatch(model, water.lattice_positions(model, 1, 0), seed=0, warps_per_block=9)
    with pytest.raises(_lib.JfgpuError):
        batch.run(1)
    assert batch.states()[0]["events"] == 0
    empty = water.WaterBatch(model, np.zeros((0, 24, 3)), seed=0)
    assert empty.run(5, record=True).shape == (0, 5)
