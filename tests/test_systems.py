"""Seeded initial states (CPU): random sequential addition on a cell grid (host code of libjfgpu.so)."""
import numpy as np
import pytest

from jellyfysh_gb300 import systems


def _min_distance(positions, length):
    d = positions[:, None, :] - positions[None, :, :]
    d -= length * np.round(d / length)
    r = np.sqrt((d ** 2).sum(-1))
    np.fill_diagonal(r, np.inf)
    return r.min()


@pytest.mark.parametrize("n, fraction", [(1, 0.1), (40, 0.3), (700, 0.2), (1500, 0.34)])
def test_grid_random_sequential_addition_places_non_overlapping_spheres(n, fraction):
    radius = 0.5
    length = systems.hard_sphere_box(n, fraction, radius)
    positions = systems.random_sequential_addition_grid(n, radius, length, seed=11)
    assert positions.shape == (n, 3)
    assert (positions >= 0.0).all() and (positions < length).all()
    if n > 1:
        assert _min_distance(positions, length) >= 2.0 * radius
    again = systems.random_sequential_addition_grid(n, radius, length, seed=11)
    assert np.array_equal(positions, again)
    other = systems.random_sequential_addition_grid(n, radius, length, seed=12)
    assert not np.array_equal(positions, other)


def test_grid_random_sequential_addition_gives_up_beyond_jamming():
    radius = 0.5
    length = systems.hard_sphere_box(200, 0.6, radius)  # far above the jamming density of the addition (~0.38)
    with pytest.raises(RuntimeError):
        systems.random_sequential_addition_grid(200, radius, length, seed=1, max_trials=100_000)
