"""The batched configurations of the path on the GPU against the oracle, event by event.

* Batched hard spheres (chains of the batched workload): per chain the packing fraction drawn from [0.10, 0.45] and
  N from {32 .. 2048}, started by random sequential addition below 0.35 and from a jittered face-centred cubic
  lattice (±2 % of the spacing) above (N = 4 k^3 there, whole lattice cells), chain length 0.3 L, cells of at least
  one diameter: every event of the FP64 path equals the oracle's bit for bit, and the mixed path equals it too.
* Batched Coulomb replicas: 32 point charges (16 of each sign) with a hard core of radius 0.05 in the unit cube,
  beta = 1, merged-image Coulomb (alpha = 3.45, real-space images to |n| <= 2, k-vectors to |k| <= 6) bounded by
  the inverse-power bound, cell veto on 8^3 cells: discrete outcomes equal the oracle's, event times to 1e-12
  relative, positions to 1e-12 of the box.
"""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DISCRETE = ("kind", "moved", "target", "new_active", "new_direction", "accepted")


def test_batched_hard_spheres_against_the_oracle():
    from jellyfysh_gb300 import ChainBatch, chain_key, workloads
    # the batched hard-sphere workload itself, 32 of its chains: N from 32 to 2048, packing fractions 0.10 - 0.45
    specs, positions, _, _ = workloads.hard_spheres(32, seed_offset=7)
    sizes = np.array([spec.n for spec in specs])
    fractions = np.array([spec.n * (4.0 / 3.0) * np.pi * spec.hs_radius ** 3 / spec.system_length ** 3
                          for spec in specs])
    assert sizes.max() > 1500 and sizes.min() < 300
    assert fractions.max() > 0.4 and fractions.min() < 0.15
    events = 300
    batch = ChainBatch(specs, positions, seed=8)
    logs = batch.run(events, mode="exact", log_capacity=events)
    batch.check_status()
    mixed = ChainBatch(specs, positions, seed=8)
    mixed_logs = mixed.run(events, mode="mixed", log_capacity=events)
    mixed.check_status()
    for c, spec in enumerate(specs):
        system = oracle.make_system(n=spec.n, system_length=spec.system_length, cells_per_side=spec.cells_per_side,
                                    neighbor_layers=spec.neighbor_layers, max_occupants=1, chain_time=spec.chain_time,
                                    initial_active=spec.initial_active, initial_direction=spec.initial_direction,
                                    potential=oracle.POT_HARD_SPHERE, hs_radius=spec.hs_radius,
                                    rng_key=chain_key(8, c))
        chain = oracle.Chain(system, positions[c])
        expected = chain.run(events)
        for field in expected.dtype.names:
            assert np.array_equal(logs[c][field], expected[field]), (c, field)
            assert np.array_equal(mixed_logs[c][field], expected[field]), (c, field)
        assert np.array_equal(batch.positions(c), chain.positions())
        assert np.array_equal(mixed.positions(c), chain.positions())
    batch.close()
    mixed.close()


def test_batched_coulomb_replicas_against_the_oracle():
    from jellyfysh_gb300 import ChainBatch, ChainSpec, chain_key, systems
    rng = np.random.default_rng(44)
    n, replicas, events = 32, 6, 400
    charges = systems.alternating_charges(n)
    specs, positions = [], []
    for c in range(replicas):
        specs.append(ChainSpec(n=n, system_length=1.0, cells_per_side=8, neighbor_layers=1, potential="coulomb",
                               far="cell_veto", hs_radius=0.05, beta=1.0, chain_time=0.7, coulomb_prefactor=1.0,
                               bound_prefactor=1.5837, ewald_alpha=3.45, fourier_cutoff=6, position_cutoff=2,
                               estimator_points=4, estimator_prefactor=1.0, initial_active=int(rng.integers(n)),
                               initial_direction=int(rng.integers(3))))
        positions.append(systems.random_sequential_addition(n, 0.05, 1.0, rng))
    batch = ChainBatch(specs, positions, [charges] * replicas, seed=9)
    logs = batch.run(events, mode="exact", log_capacity=events)
    batch.check_status()
    mixed = ChainBatch(specs, positions, [charges] * replicas, seed=9)
    mixed_logs = mixed.run(events, mode="mixed", log_capacity=events)
    mixed.check_status()
    for c, spec in enumerate(specs):
        system = oracle.make_system(n=n, system_length=1.0, cells_per_side=8, neighbor_layers=1, max_occupants=1,
                                    beta=1.0, chain_time=0.7, initial_active=spec.initial_active,
                                    initial_direction=spec.initial_direction, potential=oracle.POT_COULOMB,
                                    hs_radius=0.05, coulomb_prefactor=1.0, bound_prefactor=1.5837, ewald_alpha=3.45,
                                    fourier_cutoff=6, position_cutoff=2, far=oracle.FAR_CELL_VETO,
                                    estimator_points=4, estimator_prefactor=1.0, rng_key=chain_key(9, c))
        chain = oracle.Chain(system, positions[c], charges)
        expected = chain.run(events)
        for field in DISCRETE:
            assert np.array_equal(logs[c][field], expected[field]), (c, field)
        t_gpu = logs[c]["time_q"] + logs[c]["time_r"]
        t_cpu = expected["time_q"] + expected["time_r"]
        assert np.allclose(t_gpu, t_cpu, rtol=1e-12, atol=0.0), c
        assert np.allclose(batch.positions(c), chain.positions(), rtol=0.0, atol=1e-12)
        for field in logs.dtype.names:
            assert np.array_equal(mixed_logs[c][field], logs[c][field]), (c, field)
    batch.close()
    mixed.close()


def test_coulomb_null_veto_runs_in_pieces_with_stop_times():
    """The Coulomb kernel commits runs of null cell-veto events together.  Calls of a few events (runs cut by the
    event budget), stop times inside runs and long calls (runs cut by thinnings and by the veto window) give the
    events, the whole chain state and the positions of the FP64 path bit for bit."""
    from jellyfysh_gb300 import ChainBatch, ChainSpec, systems
    rng = np.random.default_rng(45)
    n, replicas = 32, 8
    charges = systems.alternating_charges(n)
    specs, positions = [], []
    for c in range(replicas):
        specs.append(ChainSpec(n=n, system_length=1.0, cells_per_side=8, neighbor_layers=1, potential="coulomb",
                               far="cell_veto", hs_radius=0.05, beta=1.0, chain_time=0.7, coulomb_prefactor=1.0,
                               bound_prefactor=1.5837, ewald_alpha=3.45, fourier_cutoff=6, position_cutoff=2,
                               estimator_points=4, estimator_prefactor=1.0, initial_active=int(rng.integers(n)),
                               initial_direction=int(rng.integers(3))))
        positions.append(systems.random_sequential_addition(n, 0.05, 1.0, rng))
    calls = [(3, None), (7, None), (200, 0.37), (1, None), (40, 0.81), (300, None), (5, 1.9), (500, None)]
    results = {}
    for mode in ("exact", "mixed"):
        batch = ChainBatch(specs, positions, [charges] * replicas, seed=12)
        logs = [batch.run(events, stop_time=stop, mode=mode, log_capacity=events) for events, stop in calls]
        batch.check_status()
        results[mode] = (logs, batch.state(), batch.positions())
        batch.close()
    (exact_logs, exact_state, exact_pos), (mixed_logs, mixed_state, mixed_pos) = results["exact"], results["mixed"]
    for a, b in zip(exact_logs, mixed_logs):
        for field in a.dtype.names:
            assert np.array_equal(a[field], b[field]), field
    # the chain itself; the counters of screened and re-solved candidates count different work in the two paths
    for field in ("time_q", "time_r", "eoc_q", "eoc_r", "events", "active", "direction", "eoc_new_active",
                  "occ_active", "occ_cell", "n_surplus", "status", "stopped", "lift_sum", "liftings"):
        assert np.array_equal(exact_state[field], mixed_state[field]), field
    assert np.array_equal(exact_pos, mixed_pos)
    assert (exact_state["events"] > 600).all()
