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
