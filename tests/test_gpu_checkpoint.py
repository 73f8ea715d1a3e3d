"""Checkpoint and resume of a chain batch on the GPU (the reference dumps and resumes its mediator with dill,
``output_handler/dumping_output_handler.py:70-90``, ``resume.py:63-105``): a batch restored from a checkpoint
continues bit for bit like the batch that was never interrupted, in both precisions."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["exact", "mixed"])
def test_restored_batch_continues_bit_for_bit(tmp_path, mode):
    from jellyfysh_gb300 import ChainBatch, ChainSpec, systems
    rng = np.random.default_rng(12)
    n = 64
    length = systems.lennard_jones_box(n, 0.8)
    specs = [ChainSpec(n=n, system_length=length, cells_per_side=4, potential="lennard_jones", far="cell_bounding",
                       beta=1.0 / 1.2, chain_time=2.0, initial_active=int(rng.integers(n)),
                       initial_direction=int(rng.integers(3))) for _ in range(16)]
    hs_length = systems.hard_sphere_box(200, 0.3, radius=0.5)
    specs += [ChainSpec(n=200, system_length=hs_length, cells_per_side=6, max_occupants=2, hs_radius=0.5,
                        chain_time=0.3 * hs_length, initial_active=3, initial_direction=1) for _ in range(4)]
    positions = [systems.simple_cubic_jitter(n, length, 0.05, rng) for _ in range(16)]
    positions += [systems.random_sequential_addition(200, 0.5, hs_length, rng) for _ in range(4)]
    batch = ChainBatch(specs, positions, seed=21)
    batch.run(150, mode=mode)
    path = str(tmp_path / "batch.npz")
    batch.checkpoint(path)
    batch.run(150, mode=mode)
    batch.check_status()
    restored = ChainBatch.restore(path)
    restored.run(150, mode=mode)
    restored.check_status()
    for c in range(len(specs)):
        assert np.array_equal(batch.positions(c), restored.positions(c)), c
        assert np.array_equal(batch.occupancy(c), restored.occupancy(c)), c
    original, again = batch.state(), restored.state()
    for field in original.dtype.names:
        assert np.array_equal(original[field], again[field]), field
    batch.close()
    restored.close()


def test_mirror_refresh_rebuilds_the_fp32_mirror_from_uploaded_positions():
    from jellyfysh_gb300 import ChainBatch, ChainSpec, systems
    rng = np.random.default_rng(2)
    n = 64
    length = systems.lennard_jones_box(n, 0.8)
    specs = [ChainSpec(n=n, system_length=length, cells_per_side=4, potential="lennard_jones", far="cell_veto",
                       beta=1.0 / 1.2, chain_time=2.0) for _ in range(3)]
    batch = ChainBatch(specs, [systems.simple_cubic_jitter(n, length, 0.05, rng) for _ in range(3)], seed=4)
    batch.run(100, mode="mixed")
    mirror = batch.positions32_dev.clone()
    batch.positions32_dev.zero_()
    batch.refresh_mirror()
    assert torch.equal(batch.positions32_dev, mirror)  # the engine's mirror is exactly float(positions)
    expected = batch.positions_dev[n:2 * n].to(torch.float32)
    batch.positions32_dev.zero_()
    batch.refresh_mirror(first=1, count=1)
    assert torch.equal(batch.positions32_dev[n:2 * n, :3], expected)
    assert not batch.positions32_dev[:n].any() and not batch.positions32_dev[2 * n:].any()
    batch.close()


@pytest.mark.parametrize("groups", [1, 2])
def test_rewound_batch_with_far_ahead_records(groups):
    """The far units' small keyed draws of every chain's next event are listed in records that the engine keeps
    between calls.  A batch of uniform cell-bounding Lennard-Jones chains rewound in place to an earlier state (its
    records then name later events), advanced with stop times and in chain groups, gives the FP64 path's chains bit
    for bit."""
    from jellyfysh_gb300 import ChainBatch, ChainSpec, systems
    rng = np.random.default_rng(31)
    n = 64
    length = systems.lennard_jones_box(n, 0.8)
    specs = [ChainSpec(n=n, system_length=length, cells_per_side=4, potential="lennard_jones", far="cell_bounding",
                       beta=1.0 / 1.2, chain_time=2.0, initial_active=int(rng.integers(n)),
                       initial_direction=int(rng.integers(3))) for _ in range(64)]
    positions = [systems.simple_cubic_jitter(n, length, 0.05, rng) for _ in range(64)]
    mixed = ChainBatch(specs, positions, seed=33)
    mixed.set_groups(groups)
    mixed.run(100, mode="mixed")
    saved = [t.clone() for t in mixed.state_tensors()]
    mixed.run(60, mode="mixed")
    for target, source in zip(mixed.state_tensors(), saved):
        target.copy_(source)
    mixed.run(40, stop_time=3.5, mode="mixed")
    mixed.run(120, mode="mixed")
    mixed.check_status()
    exact = ChainBatch(specs, positions, seed=33)
    exact.run(100, mode="exact")
    exact.run(40, stop_time=3.5, mode="exact")
    exact.run(120, mode="exact")
    exact.check_status()
    for c in range(len(specs)):
        assert np.array_equal(mixed.positions(c), exact.positions(c)), c
    a, b = mixed.state(), exact.state()
    for field in ("time_q", "time_r", "eoc_q", "eoc_r", "events", "active", "direction", "eoc_new_active",
                  "occ_active", "occ_cell", "n_surplus", "status", "stopped", "lift_sum", "liftings"):
        assert np.array_equal(a[field], b[field]), field
    mixed.close()
    exact.close()
