"""Seeded synthetic initial states of the benchmark and parity systems.

The reference draws random positions without overlap rejection and gives every atom the same charge
(``input_output_handler/input_handler/random_node_creator/atom_random_node_creator.py:56-67``), so the states
here are generated directly: random sequential addition for hard spheres and point charges with a hard core,
simple-cubic and face-centred-cubic lattices with uniform jitter for dense systems.  All generators take a
``numpy.random.Generator`` and return float64 arrays of shape ``(n, 3)`` with every coordinate in ``[0, L)``.
"""
import math
from typing import Optional

import numpy as np


def _wrap(positions: np.ndarray, system_length: float) -> np.ndarray:
    positions = np.mod(positions, system_length)
    positions[positions >= system_length] = 0.0
    return positions


def random_sequential_addition(n: int, radius: float, system_length: float, rng: np.random.Generator,
                               max_trials: int = 10_000_000) -> np.ndarray:
    """Uniform trial points; a trial closer than ``2 * radius`` (minimum image) to a placed sphere is rejected."""
    diameter_sq = (2.0 * radius) ** 2
    placed = np.zeros((n, 3), dtype=np.float64)
    count = 0
    trials = 0
    batch = 256
    while count < n:
        candidates = rng.uniform(0.0, system_length, size=(batch, 3))
        for candidate in candidates:
            trials += 1
            if trials > max_trials:
                raise RuntimeError("random sequential addition did not place %d spheres" % n)
            if count:
                separation = placed[:count] - candidate
                separation -= system_length * np.round(separation / system_length)
                if np.min(np.einsum("ij,ij->i", separation, separation)) < diameter_sq:
                    continue
            placed[count] = candidate
            count += 1
            if count == n:
                break
    return _wrap(placed, system_length)


def random_sequential_addition_grid(n: int, radius: float, system_length: float, seed: int,
                                    max_trials: int = 200_000_000) -> np.ndarray:
    """Random sequential addition as ``random_sequential_addition``, with the trial points from a SplitMix64 stream of
    ``seed`` and the overlap test over a cell grid (host code of libjfgpu.so): thousands of spheres near the jamming
    density in milliseconds."""
    from . import _lib
    positions = np.zeros((n, 3), dtype=np.float64)
    code = _lib.load_library().jfgpu_random_sequential_addition(int(n), float(radius), float(system_length),
                                                                 int(seed) & ((1 << 64) - 1), int(max_trials),
                                                                 positions.ctypes.data)
    if code != 0:
        raise RuntimeError("random sequential addition did not place %d spheres of radius %r in a box of %r"
                           % (n, radius, system_length))
    return _wrap(positions, system_length)


def simple_cubic_jitter(n: int, system_length: float, jitter: float, rng: np.random.Generator) -> np.ndarray:
    """First ``n`` sites (lexicographic order) of an ``m^3`` simple-cubic lattice, ``m = ceil(n^(1/3))``, plus a
    uniform jitter in ``[-jitter, jitter]`` per coordinate."""
    m = int(math.ceil(round(n ** (1.0 / 3.0), 9)))
    while m ** 3 < n:
        m += 1
    spacing = system_length / m
    grid = np.stack(np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij"), axis=-1).reshape(-1, 3)
    sites = (grid[:n].astype(np.float64) + 0.5) * spacing
    sites += rng.uniform(-jitter, jitter, size=sites.shape)
    return _wrap(sites, system_length)


def fcc_jitter(n: int, system_length: float, jitter_fraction: float, rng: np.random.Generator) -> np.ndarray:
    """First ``n`` sites of a face-centred-cubic lattice of ``k^3`` cubic cells, ``k = ceil((n/4)^(1/3))``, plus a
    uniform jitter of ``+-jitter_fraction`` of the nearest-neighbour spacing per coordinate."""
    k = max(1, int(math.ceil(round((n / 4.0) ** (1.0 / 3.0), 9))))
    while 4 * k ** 3 < n:
        k += 1
    a = system_length / k
    basis = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]])
    grid = np.stack(np.meshgrid(np.arange(k), np.arange(k), np.arange(k), indexing="ij"), axis=-1).reshape(-1, 3)
    sites = (grid[:, None, :] + basis[None, :, :]).reshape(-1, 3)[:n] * a + 0.25 * a
    spacing = a / math.sqrt(2.0)
    sites = sites + rng.uniform(-jitter_fraction * spacing, jitter_fraction * spacing, size=sites.shape)
    return _wrap(sites, system_length)


def alternating_charges(n: int) -> np.ndarray:
    """Charges +1, -1, +1, ... (``n/2`` of each sign for even ``n``)."""
    charges = np.ones(n, dtype=np.float64)
    charges[1::2] = -1.0
    return charges


def hard_sphere_box(n: int, packing_fraction: float, radius: float = 1.0) -> float:
    """Side of the cubic box holding ``n`` spheres of ``radius`` at ``packing_fraction``."""
    return (n * 4.0 / 3.0 * math.pi * radius ** 3 / packing_fraction) ** (1.0 / 3.0)


def lennard_jones_box(n: int, density: float, sigma: float = 1.0) -> float:
    return (n / density) ** (1.0 / 3.0) * sigma


def min_image_min_distance(positions: np.ndarray, system_length: float, limit: Optional[int] = None) -> float:
    """Smallest minimum-image pair distance (for checks of generated states)."""
    p = positions if limit is None else positions[:limit]
    best = math.inf
    for i in range(len(p) - 1):
        s = p[i + 1:] - p[i]
        s -= system_length * np.round(s / system_length)
        best = min(best, float(np.sqrt(np.min(np.einsum("ij,ij->i", s, s)))))
    return best


def batched_hard_sphere_state(n: int, packing_fraction: float, radius: float, rng: np.random.Generator,
                              rsa_limit: float = 0.35, fcc_jitter_fraction: float = 0.02):
    """A start of the batched hard-sphere workload: random sequential addition below ``rsa_limit``, a face-centred
    cubic lattice with a uniform jitter of ``fcc_jitter_fraction`` of the nearest-neighbour spacing above it.
    Returns (positions, system length)."""
    length = hard_sphere_box(n, packing_fraction, radius)
    if packing_fraction < rsa_limit:
        return random_sequential_addition(n, radius, length, rng), length
    # a partly filled lattice of k^3 cells is compressed into the box: it must still keep the spheres apart
    k = max(1, int(math.ceil(round((n / 4.0) ** (1.0 / 3.0), 9))))
    spacing = length / k / math.sqrt(2.0)
    if spacing * (1.0 - 2.0 * fcc_jitter_fraction) < 2.0 * radius:
        raise ValueError("n = %d spheres at packing fraction %.3f overlap on a partly filled fcc lattice of %d^3 "
                         "cells; take n = 4 k^3" % (n, packing_fraction, k))
    return fcc_jitter(n, length, fcc_jitter_fraction, rng), length



def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """A uniformly random rotation matrix (unit quaternion from four normal deviates)."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def water_lattice(molecules_per_side: int, system_length: float, oh_length: float, hh_length: float,
                  rng: np.random.Generator, charge_oxygen: float = -0.82, charge_hydrogen: float = 0.41):
    """Water molecules on a simple-cubic lattice of ``molecules_per_side``^3 sites (site centres ``(i + 1/2) L / m``)
    in seeded uniformly random orientations; the bonds have the equilibrium lengths (O–H and H–H, hence the angle).
    As the reference's water node creator does (``water_random_node_creator.py``), the site is the molecule's
    barycentre of equal weights, so that the oxygens are off the lattice lines.  Leaf units in the reference's order
    per molecule, hydrogen, oxygen, hydrogen.  Returns (positions [3 m^3][3] in [0, L), charges [3 m^3])."""
    half_angle = math.asin(hh_length / (2.0 * oh_length))
    bond_one = np.array([math.sin(half_angle), math.cos(half_angle), 0.0]) * oh_length
    bond_two = np.array([-math.sin(half_angle), math.cos(half_angle), 0.0]) * oh_length
    spacing = system_length / molecules_per_side
    positions = []
    for iz in range(molecules_per_side):
        for iy in range(molecules_per_side):
            for ix in range(molecules_per_side):
                centre = (np.array([ix, iy, iz], dtype=np.float64) + 0.5) * spacing
                rotation = random_rotation(rng)
                one, two = rotation @ bond_one, rotation @ bond_two
                oxygen = centre - (one + two) / 3.0
                positions.extend([oxygen + one, oxygen, oxygen + two])
    molecules = molecules_per_side ** 3
    charges = np.tile(np.array([charge_hydrogen, charge_oxygen, charge_hydrogen]), molecules)
    return _wrap(np.array(positions, dtype=np.float64), system_length), charges


def water_roots(positions: np.ndarray, system_length: float) -> np.ndarray:
    """The root unit of every water molecule (leaf units hydrogen, oxygen, hydrogen): the oxygen plus the mean of the
    two O–H bond vectors taken in the minimum image, wrapped into [0, L).  Computed in Python floats component by
    component, as the reference's water node creator places the barycentre
    (``water_random_node_creator.py:83-99``: the oxygen is the centre minus the mean of the two bonds).
    positions [3 M][3] -> roots [M][3]."""
    length = float(system_length)
    half = length / 2.0
    atoms = np.asarray(positions, dtype=np.float64).reshape(-1, 3, 3).tolist()
    roots = []
    for hydrogen_one, oxygen, hydrogen_two in atoms:
        centre = []
        for d in range(3):
            one = ((hydrogen_one[d] - oxygen[d]) + half) % length - half
            two = ((hydrogen_two[d] - oxygen[d]) + half) % length - half
            centre.append((oxygen[d] + (one + two) / 3.0) % length)
        roots.append(centre)
    return np.array(roots, dtype=np.float64).reshape(-1, 3)
