"""The batched solve of the GPU neighbourhood event handler against the oracle (GPU; no reference tree needed).

``GpuNeighbourhoodEventHandler`` (``plugin/event_handler``) solves the pair events of the active unit against every
target of its neighbourhood with one launch of the GPU potential's ``displacements`` and takes the earliest
(``plugin/potential/_common.py``: ``earliest``).  On random neighbourhoods (velocities along one positive axis,
separations in the periodic box, charges of either sign, potential changes from the keyed draws) the earliest target
and its time equal those of the oracle's per-pair solves (pinned to the reference's potentials by
``tests/test_oracle_known_answers.py``): the target exactly, the time to 1e-12 relative (hard spheres bit for bit).
The handler's wiring inside the reference's own mediator is tested by ``tests/test_plugin.py`` (with a reference tree).
"""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REL = 1e-12


def _neighbourhoods(rng, count, length):
    for _ in range(count):
        n = int(rng.integers(1, 300))
        velocity = [0.0, 0.0, 0.0]
        velocity[int(rng.integers(3))] = float(rng.uniform(0.5, 2.0))
        separations = rng.uniform(-0.5 * length, 0.5 * length, (n, 3))
        charges = rng.choice([-1.0, 1.0], (n, 2))
        changes = [oracle.expovariate(oracle.draw(97, e, oracle.RNG_PAIR, j), 1.0) for e, j in
                   zip(rng.integers(0, 1 << 20, n), range(n))]
        yield velocity, separations, charges, changes


def _earliest_oracle(times):
    index = int(np.argmin(times))
    return (-1, float("inf")) if np.isinf(times[index]) else (index, float(times[index]))


def _check(potential, solve_one, length, seed, exact_bits=False, count=40):
    from jellyfysh_gb300.plugin.potential._common import earliest
    rng = np.random.default_rng(seed)
    hits = 0
    for velocity, separations, charges, changes in _neighbourhoods(rng, count, length):
        expected = []
        for s, c, du in zip(separations, charges, changes):
            try:
                expected.append(solve_one(velocity, s, c, du))
            except oracle.OracleError:
                expected.append(None)
        if any(t is None for t in expected):
            with pytest.raises(Exception):
                earliest(potential, velocity, separations, charges, changes)
            continue
        index, time = earliest(potential, velocity, separations, charges, changes)
        want_index, want_time = _earliest_oracle(np.array(expected))
        assert index == want_index
        if index >= 0:
            hits += 1
            if exact_bits:
                assert time == want_time
            else:
                assert abs(time - want_time) <= REL * abs(want_time)
    assert hits > count // 4


def test_earliest_pair_of_hard_spheres():
    from jellyfysh_gb300.plugin.potential.gpu_hard_sphere_potential import GpuHardSpherePotential
    radius = 0.05
    potential = GpuHardSpherePotential(radius)
    rng = np.random.default_rng(1)
    from jellyfysh_gb300.plugin.potential._common import earliest
    hits = 0
    for _ in range(40):
        n = int(rng.integers(1, 300))
        velocity = [0.0, 0.0, 0.0]
        velocity[int(rng.integers(3))] = 1.0
        separations = rng.uniform(-0.5, 0.5, (n, 3))
        norms = np.linalg.norm(separations, axis=1)
        separations = separations[norms > 2.0 * radius]  # hard spheres do not overlap
        expected = np.array([oracle.hs_displacement(radius, velocity, s) for s in separations])
        index, time = earliest(potential, velocity, separations, None, None)
        want_index, want_time = _earliest_oracle(expected) if len(expected) else (-1, float("inf"))
        assert index == want_index
        if index >= 0:
            hits += 1
            assert time == want_time
    assert hits > 5


def test_earliest_pair_of_lennard_jones():
    from jellyfysh_gb300.plugin.potential.gpu_lennard_jones_potential import GpuLennardJonesPotential
    potential = GpuLennardJonesPotential(1.0, 1.0)
    length = 10.857670466379625
    _check(potential, lambda v, s, c, du: oracle.lj_displacement(1.0, 1.0, v, s, du), length, seed=2)


def test_earliest_pair_of_inverse_power_charges():
    from jellyfysh_gb300.plugin.potential.gpu_inverse_power_potential import GpuInversePowerPotential
    potential = GpuInversePowerPotential(1.0, 1.0)
    _check(potential, lambda v, s, c, du: oracle.ip_displacement(1.0, 1.0, v, s, c[0], c[1], du), 1.0, seed=3)


def test_earliest_pair_of_displaced_even_power_bonds():
    from jellyfysh_gb300.plugin.potential.gpu_displaced_even_power_potential import GpuDisplacedEvenPowerPotential
    potential = GpuDisplacedEvenPowerPotential(0.3, 2, 5.0)
    _check(potential, lambda v, s, c, du: oracle.dep_displacement(0.3, 2, 5.0, v, s, du), 1.0, seed=4)


def test_earliest_pair_of_the_coulomb_bound():
    from jellyfysh_gb300.plugin.potential.gpu_inverse_power_coulomb_bounding_potential import \
        GpuInversePowerCoulombBoundingPotential
    potential = GpuInversePowerCoulombBoundingPotential(1.5837)
    potential._system_length = 1.0  # the box of the setting (no reference setting in this test)
    _check(potential, lambda v, s, c, du: oracle.ipcb_displacement(1.5837, 1.0, v, s, c[0], c[1], du), 1.0,
           seed=5)
