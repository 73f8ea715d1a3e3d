"""The batched workloads of the event-time path: chain parameters and seeded synthetic initial states.

Each builder returns ``(specs, positions, charges, system_length)`` for ``ChainBatch`` (``charges`` is None for
uncharged systems).  The parameters are those of the reference's vocabulary (INI sections of
``jellyfysh/potential``, ``jellyfysh/event_handler``, ``jellyfysh/activator``):

* ``lennard_jones``: N = 1024 Lennard-Jones atoms (epsilon = sigma = 1) at density 0.8, beta = 1/1.2, 12^3 cells with
  three neighbour layers (the nearby cells cover the 2.5 sigma cutoff), far field by the cell-bounding potential
  (InnerPointEstimator bounds, prefactor 1.5, 10 points per side), chain time 2 sigma, seeded simple-cubic lattice
  plus +-0.05 sigma jitter.
* ``coulomb``: 32 point charges (16 of each sign) with a hard core of radius 0.05 in the unit cube, beta = 1,
  merged-image Coulomb (alpha = 3.45, |n| <= 2, |k| <= 6) bounded by the inverse-power Coulomb bound, cell veto on
  8^3 cells, seeded random sequential addition.
* ``hard_spheres``: independent hard-sphere chains of uneven size and density (N drawn from 32..2048, packing
  fraction from [0.10, 0.45]; random sequential addition below 0.35, a jittered fcc lattice above), cells whose
  nearby cells reach one diameter and fit with one more cell in half the box, chain time 0.3 L.
* ``hard_spheres_n64``: N = 64 spheres of radius 0.1 in the unit cube, 5^3 cells, chain time 0.3.
"""
import numpy as np

from . import systems
from .chains import ChainSpec

LENNARD_JONES = dict(workload="lennard_jones_chains_4096x1024_cell_bounding", chains=4096, n=1024, density=0.8,
                     beta=1.0 / 1.2, cells_per_side=12, neighbor_layers=3, chain_time=2.0, far="cell_bounding",
                     jitter=0.05, estimator_points=10, estimator_prefactor=1.5)
COULOMB = dict(workload="coulomb_replicas_1024x32_cell_veto", chains=1024, n=32, hard_core_radius=0.05,
               system_length=1.0, beta=1.0, cells_per_side=8, neighbor_layers=1, chain_time=0.7,
               coulomb_prefactor=1.0, bound_prefactor=1.5837, ewald_alpha=3.45, fourier_cutoff=6, position_cutoff=2,
               far="cell_veto", estimator_points=10, estimator_prefactor=1.0)
HARD_SPHERES = dict(workload="hard_sphere_chains_4096_uneven", chains=4096, n_min=32, n_max=2048, eta_min=0.10,
                    eta_max=0.45, lattice_above=0.35, radius=0.5, chain_time_over_length=0.3)
HARD_SPHERES_N64 = dict(workload="hard_sphere_chains_n64", chains=4096, n=64, radius=0.1, system_length=1.0,
                        cells_per_side=5, chain_time=0.3)


def lennard_jones(chains, seed_offset=0, n=None):
    """The batched Lennard-Jones workload (``n`` atoms per chain, 1024 by default)."""
    w = LENNARD_JONES
    n = w["n"] if n is None else n
    length = systems.lennard_jones_box(n, w["density"])
    rng = np.random.default_rng(1234 + seed_offset)
    specs, positions = [], []
    for _ in range(chains):
        specs.append(ChainSpec(n=n, system_length=length, cells_per_side=w["cells_per_side"],
                               potential="lennard_jones", far=w["far"], neighbor_layers=w["neighbor_layers"],
                               beta=w["beta"], chain_time=w["chain_time"], estimator_points=w["estimator_points"],
                               estimator_prefactor=w["estimator_prefactor"], initial_active=int(rng.integers(n)),
                               initial_direction=int(rng.integers(3))))
        positions.append(systems.simple_cubic_jitter(n, length, w["jitter"], rng))
    return specs, positions, None, length


def coulomb(chains, seed_offset=0):
    """Replicas of 32 point charges (16 of each sign) with a hard core in the unit cube, cell veto on 8^3 cells."""
    w = COULOMB
    rng = np.random.default_rng(4321 + seed_offset)
    specs, positions = [], []
    for _ in range(chains):
        specs.append(ChainSpec(n=w["n"], system_length=w["system_length"], cells_per_side=w["cells_per_side"],
                               neighbor_layers=w["neighbor_layers"], potential="coulomb", far=w["far"],
                               hs_radius=w["hard_core_radius"], beta=w["beta"], chain_time=w["chain_time"],
                               coulomb_prefactor=w["coulomb_prefactor"], bound_prefactor=w["bound_prefactor"],
                               ewald_alpha=w["ewald_alpha"], fourier_cutoff=w["fourier_cutoff"],
                               position_cutoff=w["position_cutoff"], estimator_points=w["estimator_points"],
                               estimator_prefactor=w["estimator_prefactor"], initial_active=int(rng.integers(w["n"])),
                               initial_direction=int(rng.integers(3))))
        positions.append(systems.random_sequential_addition(w["n"], w["hard_core_radius"], w["system_length"], rng))
    charges = [systems.alternating_charges(w["n"])] * chains
    return specs, positions, charges, w["system_length"]


def hard_sphere_cells(length, diameter):
    """(cells per side, neighbour layers) of a hard-sphere chain in a periodic cube of side ``length``: the nearby
    cells reach at least one diameter (layers x side >= diameter) and the nearby cells plus one cell fit in half the
    box ((layers + 1) x side <= length / 2), so that the minimum image of every target that the active sphere can
    reach before its next cell-boundary event is the one its candidate is solved for.  One layer where the box
    allows it (length >= 4 diameters), else the fewest layers that fit; cells as many as the layers allow, at most
    64 per side."""
    for layers in (1, 2, 3, 4):
        m = min(int(layers * length / diameter), 64)
        if m >= 2 * (layers + 1):
            return m, layers
    raise ValueError("no cell system fits a periodic cube of side %r for spheres of diameter %r"
                     % (length, diameter))


def hard_sphere_chain(n, eta, rng, radius=0.5, lattice_above=0.35, chain_time_over_length=0.3):
    """One hard-sphere chain of ``n`` spheres at packing fraction ``eta``: (spec, positions), cells from
    ``hard_sphere_cells``."""
    if eta < lattice_above:
        # random sequential addition on a cell grid (thousands of spheres near the jamming density)
        length = systems.hard_sphere_box(n, eta, radius)
        state = systems.random_sequential_addition_grid(n, radius, length, seed=int(rng.integers(1 << 62)))
    else:
        state, length = systems.batched_hard_sphere_state(n, eta, radius, rng, rsa_limit=lattice_above)
    m, layers = hard_sphere_cells(length, 2.0 * radius)
    spec = ChainSpec(n=n, system_length=length, cells_per_side=m, neighbor_layers=layers, max_occupants=1,
                     hs_radius=radius, chain_time=chain_time_over_length * length,
                     initial_active=int(rng.integers(n)), initial_direction=int(rng.integers(3)))
    return spec, state


def hard_spheres(chains, seed_offset=0, n_max=None):
    """Independent hard-sphere chains of uneven size and density: N ~ U{32..n_max} (2048 by default), packing
    fraction ~ U[0.10, 0.45].  Lattice starts take N rounded to whole fcc cells (4 k^3)."""
    w = HARD_SPHERES
    n_max = w["n_max"] if n_max is None else n_max
    rng = np.random.default_rng(5678 + seed_offset)
    specs, positions = [], []
    for _ in range(chains):
        eta = float(rng.uniform(w["eta_min"], w["eta_max"]))
        n = int(rng.integers(w["n_min"], n_max + 1))
        if eta >= w["lattice_above"]:
            k = max(2, int(round((n / 4.0) ** (1.0 / 3.0))))
            while 4 * k ** 3 > n_max:
                k -= 1
            n = 4 * k ** 3
        spec, state = hard_sphere_chain(n, eta, rng, w["radius"], w["lattice_above"], w["chain_time_over_length"])
        specs.append(spec)
        positions.append(state)
    length = max(spec.system_length for spec in specs)
    return specs, positions, None, length


def hard_spheres_n64(chains, seed_offset=0):
    """N = 64 spheres of radius 0.1 in the unit cube by random sequential addition, 5^3 cells, chain time 0.3."""
    w = HARD_SPHERES_N64
    rng = np.random.default_rng(2468 + seed_offset)
    specs, positions = [], []
    for _ in range(chains):
        specs.append(ChainSpec(n=w["n"], system_length=w["system_length"], cells_per_side=w["cells_per_side"],
                               hs_radius=w["radius"], chain_time=w["chain_time"],
                               initial_active=int(rng.integers(w["n"])), initial_direction=int(rng.integers(3))))
        positions.append(systems.random_sequential_addition(w["n"], w["radius"], w["system_length"], rng))
    return specs, positions, None, w["system_length"]


BUILDERS = {"lennard_jones": (LENNARD_JONES, lennard_jones), "coulomb": (COULOMB, coulomb),
            "hard_spheres": (HARD_SPHERES, hard_spheres), "hard_spheres_n64": (HARD_SPHERES_N64, hard_spheres_n64)}


def near_cells(spec):
    """Nearby cells scanned per event (distinct cells within the neighbour layers)."""
    per_axis = min(2 * spec.neighbor_layers + 1, spec.cells_per_side)
    return per_axis ** 3

