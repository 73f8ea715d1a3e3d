"""The GPU event loop against the reference's trajectories, the oracle, and itself across precisions.

* Reference trajectories (``golden/trajectory_*.npz``): the FP64 path reproduces every event's kind, moved unit,
  target, lifting outcome and new direction exactly, the event times to 1e-12 relative and the committed positions
  to 1e-12 of the box; hard spheres (square roots only) bit for bit.
* Mixed precision (FP32 screening, FP64 refinement) reproduces the FP64 path bit for bit: same winners, same times.
* Random systems beyond the fixtures (two occupants per cell, two neighbour layers, heterogeneous batches) against
  the oracle.
"""
import numpy as np
import pytest

import oracle
from tests.trajectory_cases import load_trajectory, oracle_system, trajectory_names

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DISCRETE = ("kind", "moved", "target", "new_active", "new_direction", "accepted")
REL = 1e-12


def spec_from_fixture(spec):
    from jellyfysh_gb300 import ChainSpec
    return ChainSpec(n=spec["n"], system_length=spec["system_length"], cells_per_side=spec["cells_per_side"],
                     potential=spec["potential"], far=spec["far"], neighbor_layers=spec["neighbor_layers"],
                     max_occupants=1, beta=spec["beta"], chain_time=spec["chain_time"], speed=1.0,
                     hs_radius=spec.get("radius", 0.0), estimator_points=spec.get("estimator_points", 10),
                     estimator_prefactor=spec.get("estimator_prefactor", 1.5), rng_key=spec["rng_key"])


def run_fixture(name, mode):
    from jellyfysh_gb300 import ChainBatch
    spec, initial, charges, events, final = load_trajectory(name)
    batch = ChainBatch([spec_from_fixture(spec)], [initial], None if charges is None else [charges])
    log = batch.run(len(events), mode=mode, log_capacity=len(events))[0]
    batch.check_status()
    positions = batch.positions(0)
    batch.close()
    return spec, events, final, log, positions


def compare_logs(log, events, length, exact_bits):
    assert len(log) == len(events)
    for field in DISCRETE:
        bad = np.nonzero(log[field] != events[field])[0]
        assert bad.size == 0, (field, int(bad[0]), log[bad[0]], events[bad[0]])
    t_gpu = log["time_q"] + log["time_r"]
    t_ref = events["time_q"] + events["time_r"]
    assert np.all(np.abs(t_gpu - t_ref) <= REL * np.maximum(np.abs(t_ref), 1.0))
    for axis in ("x", "y", "z"):
        diff = np.abs(log[axis] - events[axis])
        diff = np.minimum(diff, length - diff)  # periodic
        assert np.all(diff <= REL * length), (axis, float(diff.max()))
    if exact_bits:
        for field in events.dtype.names:
            assert np.array_equal(log[field], events[field]), field


@pytest.mark.parametrize("name", trajectory_names())
def test_fp64_path_reproduces_reference_trajectory(name):
    spec, events, final, log, positions = run_fixture(name, "exact")
    compare_logs(log, events, spec["system_length"], exact_bits=spec["potential"] == "hard_sphere")
    diff = np.abs(positions - final)
    diff = np.minimum(diff, spec["system_length"] - diff)
    assert diff.max() <= REL * spec["system_length"]


@pytest.mark.parametrize("name", trajectory_names())
def test_mixed_precision_equals_fp64_path(name):
    _, _, _, exact_log, exact_positions = run_fixture(name, "exact")
    _, _, _, mixed_log, mixed_positions = run_fixture(name, "mixed")
    for field in exact_log.dtype.names:
        assert np.array_equal(mixed_log[field], exact_log[field]), field
    assert np.array_equal(mixed_positions, exact_positions)


def _lj_batch_inputs(chains, n=64, density=0.8, seed=0):
    from jellyfysh_gb300 import ChainSpec, systems
    length = systems.lennard_jones_box(n, density)
    rng = np.random.default_rng(seed)
    specs, positions = [], []
    for c in range(chains):
        far = "cell_veto" if c % 2 == 0 else "cell_bounding"
        specs.append(ChainSpec(n=n, system_length=length, cells_per_side=4, potential="lennard_jones", far=far,
                               beta=1.0 / 1.2, chain_time=2.0, initial_active=int(rng.integers(n)),
                               initial_direction=int(rng.integers(3))))
        positions.append(systems.simple_cubic_jitter(n, length, 0.05, rng))
    return specs, positions


def test_batched_mixed_equals_fp64_lennard_jones():
    from jellyfysh_gb300 import ChainBatch
    specs, positions = _lj_batch_inputs(96)
    results = {}
    for mode in ("exact", "mixed"):
        batch = ChainBatch(specs, positions, seed=7)
        batch.run(1500, mode=mode)
        batch.check_status()
        results[mode] = (batch.positions(), batch.state())
        batch.close()
    for a, b in zip(results["exact"][0], results["mixed"][0]):
        assert np.array_equal(a, b)
    exact_state, mixed_state = results["exact"][1], results["mixed"][1]
    for field in ("time_q", "time_r", "events", "active", "direction", "n_surplus"):
        assert np.array_equal(exact_state[field], mixed_state[field]), field
    assert (exact_state["events"] == 1500).all()


def test_chain_groups_and_kernel_timing_leave_results_unchanged():
    """Chain groups on streams of their own, CUDA events around every launch, and plain launches instead of CUDA
    graphs change no bit of the run."""
    from jellyfysh_gb300 import ChainBatch, ChainSpec, systems
    n, chains, events = 64, 256, 300
    length = systems.lennard_jones_box(n, 0.8)
    rng = np.random.default_rng(3)
    specs = [ChainSpec(n=n, system_length=length, cells_per_side=4, potential="lennard_jones", far="cell_bounding",
                       beta=1.0 / 1.2, chain_time=2.0, initial_active=int(rng.integers(n)),
                       initial_direction=int(rng.integers(3))) for _ in range(chains)]
    positions = [systems.simple_cubic_jitter(n, length, 0.05, rng) for _ in range(chains)]
    results = {}
    for label, mode, groups, timing, graphs in (("exact", "exact", 1, False, True), ("mixed", "mixed", 1, False, True),
                                                ("grouped", "mixed", 4, True, True),
                                                ("plain", "mixed", 1, False, False),
                                                ("sampled", "mixed", 1, 7, True)):
        batch = ChainBatch(specs, positions, seed=11)
        batch.set_groups(groups)
        batch.set_graphs(graphs)
        batch.set_timing(bool(timing), stride=int(timing) or 1)
        for part in (events // 3, events // 3, events - 2 * (events // 3)):  # replays of captured segments
            batch.run(part, mode=mode)
        batch.check_status()
        results[label] = (batch.positions(), batch.state())
        if label == "grouped":
            times = batch.kernel_times()
            for kind in ("screen", "resolve"):  # the settle kernel is timed as "resolve"
                assert times[kind]["launches"] == 4 * events, (kind, times[kind])
                assert times[kind]["ms"] > 0.0
            assert times["refine"]["launches"] == 0 and times["chains"]["launches"] == 0
        if label == "sampled":  # rounds 0, 7, 14, ... of each call are timed, the others replayed from graphs
            times = batch.kernel_times()
            sampled = sum((part + 6) // 7 for part in (events // 3, events // 3, events - 2 * (events // 3)))
            assert times["screen"]["launches"] == sampled
        batch.close()
    for label in ("mixed", "grouped", "plain", "sampled"):
        for a, b in zip(results["exact"][0], results[label][0]):
            assert np.array_equal(a, b), label
        for field in ("time_q", "time_r", "events", "active", "direction", "n_surplus", "occ_cell"):
            assert np.array_equal(results["exact"][1][field], results[label][1][field]), (label, field)
    assert (results["grouped"][1]["events"] == events).all()


def _occupancy_consistent(batch, chain):
    """Every unit is in exactly one place (a cell slot, the surplus list or active), and the role words agree."""
    spec = batch.specs[chain]
    occupancy = batch.occupancy(chain)
    occ = occupancy.ravel()
    surplus = batch.surplus(chain)
    ids = list(occ[occ >= 0]) + list(surplus)
    state = batch.state()[chain]
    if state["occ_active"] >= 0:
        ids.append(int(state["occ_active"]))
    if sorted(ids) != list(range(spec.n)):
        return False
    roles = batch.roles(chain)
    m = spec.cells_per_side
    for k, j in enumerate(surplus):
        if roles[j] != (1 << 24) | k:
            return False
    for cell, slots in enumerate(occupancy):
        axes = (cell % m) | (((cell // m) % m) << 8) | ((cell // (m * m)) << 16)
        if any(roles[j] != axes for j in slots if j >= 0):
            return False
    return state["occ_active"] < 0 or roles[state["occ_active"]] == 1 << 25


def test_random_hard_sphere_systems_against_oracle():
    """Heterogeneous batch: different N, box, cell system, occupancy bound and layers per chain."""
    from jellyfysh_gb300 import ChainBatch, ChainSpec, chain_key, systems
    rng = np.random.default_rng(21)
    specs, positions = [], []
    for c in range(12):
        # boxes large enough that the nearby cells plus one cell fit in half the box (minimum image holds)
        layers = 1 + c % 2
        n = int(rng.integers(200, 600))
        eta = float(rng.uniform(0.1, 0.3))
        length = systems.hard_sphere_box(n, eta, radius=0.5)
        m = min(int(length * layers), 24)
        while length / m * layers < 1.0:
            m -= 1
        assert (layers + 1) * length / m <= length / 2
        specs.append(ChainSpec(n=n, system_length=length, cells_per_side=m, neighbor_layers=layers,
                               max_occupants=1 + c % 3, hs_radius=0.5, chain_time=0.4 * length,
                               initial_active=int(rng.integers(n)), initial_direction=int(rng.integers(3))))
        positions.append(systems.random_sequential_addition(n, 0.5, length, rng))
    events = 400
    batch = ChainBatch(specs, positions, seed=3)
    logs = batch.run(events, mode="exact", log_capacity=events)
    batch.check_status()
    for c, spec in enumerate(specs):
        system = oracle.make_system(n=spec.n, system_length=spec.system_length, cells_per_side=spec.cells_per_side,
                                    neighbor_layers=spec.neighbor_layers, max_occupants=spec.max_occupants,
                                    chain_time=spec.chain_time, initial_active=spec.initial_active,
                                    initial_direction=spec.initial_direction, potential=oracle.POT_HARD_SPHERE,
                                    hs_radius=spec.hs_radius, rng_key=chain_key(3, c))
        chain = oracle.Chain(system, positions[c])
        expected = chain.run(events)
        for field in expected.dtype.names:
            assert np.array_equal(logs[c][field], expected[field]), (c, field)
        assert np.array_equal(batch.positions(c), chain.positions())
        assert _occupancy_consistent(batch, c)
    # the mixed precision path agrees on the heterogeneous batch as well
    mixed = ChainBatch(specs, positions, seed=3)
    mixed_logs = mixed.run(events, mode="mixed", log_capacity=events)
    for c in range(len(specs)):
        for field in logs.dtype.names:
            assert np.array_equal(mixed_logs[c][field], logs[c][field]), (c, field)
        assert _occupancy_consistent(mixed, c)
    batch.close()
    mixed.close()


def test_stop_time_time_slices_like_the_oracle():
    from jellyfysh_gb300 import ChainBatch
    spec, initial, charges, events, final = load_trajectory("hard_spheres_n64")
    t_stop = float(events["time_q"][199] + events["time_r"][199]) + 1e-9
    batch = ChainBatch([spec_from_fixture(spec)], [initial])
    batch.run(100_000, stop_time=t_stop, mode="mixed")
    state = batch.state()[0]
    chain = oracle.Chain(oracle_system(spec), initial)
    chain.run(100_000, stop_time=t_stop, record=False)
    expected = chain.state()
    assert state["events"] == expected["events"] == 200
    assert (state["time_q"], state["time_r"]) == (expected["time_q"], expected["time_r"])
    assert np.array_equal(batch.positions(0), chain.positions())
    batch.close()


def test_estimator_bounds_match_the_oracle():
    from jellyfysh_gb300 import ChainBatch
    for name in ("lennard_jones_n64_cell_veto", "coulomb_n8_cell_veto"):
        spec, initial, charges, events, final = load_trajectory(name)
        batch = ChainBatch([spec_from_fixture(spec)], [initial], None if charges is None else [charges])
        upper, lower = batch.bounds(0)
        chain = oracle.Chain(oracle_system(spec), initial, charges)
        expected = chain.bounds()
        np.testing.assert_allclose(upper, expected[0], rtol=1e-12, atol=0)
        np.testing.assert_allclose(lower, expected[1], rtol=1e-12, atol=0)
        batch.close()
