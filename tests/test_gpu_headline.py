"""Parity at the geometry of the batched Lennard-Jones workload, on the GPU.

N = 1024 Lennard-Jones atoms at density 0.8 in 12^3 cells with three neighbour layers (343 nearby cells), the
cell-bounding far field (estimator of 10 points per side, prefactor 1.5), chain time 2: the chains of the
benchmarked batch, fewer of them.

* FP64 path against the oracle: every event's kind, moved unit, target, lifting outcome and new direction exactly,
  event times to 1e-12 relative, committed positions to 1e-12 of the box.
* Mixed precision (FP32 screening, FP64 re-solve of the near-winners) against the FP64 path bit for bit, with the
  far-field lookups of the units that pass the rejection by the largest far rate and the re-solve of whole events in
  FP64 (refine-list overflow) both taken: the overflow is forced on a second batch by a refine-list limit of one
  entry, which must not change a bit.
"""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DISCRETE = ("kind", "moved", "target", "new_active", "new_direction", "accepted")
REL = 1e-12


def _oracle_chain(spec, positions, key):
    system = oracle.make_system(n=spec.n, system_length=spec.system_length, cells_per_side=spec.cells_per_side,
                                neighbor_layers=spec.neighbor_layers, max_occupants=spec.max_occupants,
                                beta=spec.beta, chain_time=spec.chain_time, initial_active=spec.initial_active,
                                initial_direction=spec.initial_direction, potential=oracle.POT_LENNARD_JONES,
                                far=oracle.FAR_CELL_BOUNDING, estimator_points=spec.estimator_points,
                                estimator_prefactor=spec.estimator_prefactor, rng_key=key)
    return oracle.Chain(system, positions)


def test_fp64_path_against_the_oracle_at_the_benchmarked_geometry():
    from jellyfysh_gb300 import ChainBatch, workloads
    specs, positions, _, length = workloads.lennard_jones(8, seed_offset=17)
    events = 300
    batch = ChainBatch(specs, positions, seed=21)
    logs = batch.run(events, mode="exact", log_capacity=events)
    batch.check_status()
    for c, spec in enumerate(specs):
        chain = _oracle_chain(spec, positions[c], batch.keys[c])
        expected = chain.run(events)
        for field in DISCRETE:
            bad = np.nonzero(logs[c][field] != expected[field])[0]
            assert bad.size == 0, (c, field, int(bad[0]) if bad.size else None)
        t_gpu = logs[c]["time_q"] + logs[c]["time_r"]
        t_cpu = expected["time_q"] + expected["time_r"]
        assert np.all(np.abs(t_gpu - t_cpu) <= REL * np.maximum(np.abs(t_cpu), 1.0)), c
        diff = np.abs(batch.positions(c) - chain.positions())
        diff = np.minimum(diff, length - diff)
        assert diff.max() <= REL * length, c
    # the events of the path all occur at this geometry: pair liftings and cell-bounding events (thinned and
    # accepted), cell boundaries and ends of chain
    kinds = np.bincount(np.concatenate([log["kind"] for log in logs]), minlength=8)
    for kind in (oracle.EV_PAIR, oracle.EV_CELL_BOUNDING, oracle.EV_BOUNDARY, oracle.EV_END_OF_CHAIN):
        assert kinds[kind] > 0, kinds
    batch.close()


def _run(specs, positions, mode, events, refine_limit=None):
    from jellyfysh_gb300 import ChainBatch
    batch = ChainBatch(specs, positions, seed=23)
    if refine_limit is not None:
        batch.set_refine_limit(refine_limit)
    log = batch.run(events, mode=mode, log_capacity=events)
    batch.check_status()
    result = (log, batch.positions(), batch.state())
    batch.close()
    return result


def test_mixed_precision_equals_fp64_at_the_benchmarked_geometry():
    from jellyfysh_gb300 import workloads
    specs, positions, _, _ = workloads.lennard_jones(64, seed_offset=19)
    events = 400
    exact_log, exact_positions, exact_state = _run(specs, positions, "exact", events)
    for limit in (None, 1):
        log, got_positions, state = _run(specs, positions, "mixed", events, refine_limit=limit)
        for field in exact_log.dtype.names:
            assert np.array_equal(log[field], exact_log[field]), (limit, field)
        for a, b in zip(got_positions, exact_positions):
            assert np.array_equal(a, b), limit
        for field in ("time_q", "time_r", "eoc_q", "eoc_r", "events", "active", "direction", "n_surplus",
                      "occ_cell", "lift_sum", "liftings"):
            assert np.array_equal(state[field], exact_state[field]), (limit, field)
        # the far field rejected most units from their keyed draw alone; the others read their role words
        assert 0 < int(state["far_lookups"].sum()) < 64 * events * 1023 // 10, int(state["far_lookups"].sum())
        if limit is None:
            fallbacks = int(state["refine_fallbacks"].sum())
            assert fallbacks < state["events"].sum() // 100
        else:
            # with a one-entry refine list, every event with two or more near-winners is re-solved entirely in FP64
            assert int(state["refine_fallbacks"].sum()) > max(fallbacks, 20), int(state["refine_fallbacks"].sum())
    assert (exact_state["events"] == events).all()
