"""Estimators of long runs, on the CPU: the oracle against the reference's own long runs.

* The lifting sums (excess displacement of the pressure estimator) of the oracle equal, bit for bit, the sums
  replayed from the reference's event-by-event trajectories (``golden/trajectory_*.npz``).
* Long oracle runs reproduce the reference's estimators (``golden/estimators_*.npz``, recorded from the
  reference's event loop with its own random numbers): mean potential energy and pressure within 3 standard
  errors, the pair correlation by a chi-square within 3 standard deviations.
* The estimator functions themselves on configurations with known answers.
"""
import concurrent.futures

import numpy as np
import pytest

import oracle
from jellyfysh_gb300 import estimators
from tests.estimator_cases import compare, estimator_names, reference_estimates, sampled_estimates
from tests.trajectory_cases import load_trajectory, oracle_system, trajectory_names


def replay_liftings(spec, initial, events):
    """Sum over the accepted liftings of the separation target - active along the direction, from the reference's
    trajectory (positions of the moved unit after every event), with Python float arithmetic."""
    positions = [[float(v) for v in p] for p in initial]
    length = float(spec["system_length"])
    total, count = 0.0, 0
    for ev in events:
        moved, active = int(ev["moved"]), int(ev["new_active"])
        positions[moved] = [float(ev["x"]), float(ev["y"]), float(ev["z"])]
        if active != moved and int(ev["kind"]) != oracle.EV_END_OF_CHAIN:
            d = int(ev["new_direction"])
            total += ((positions[active][d] - positions[moved][d]) + length / 2.0) % length - length / 2.0
            count += 1
    return total, count


@pytest.mark.parametrize("name", trajectory_names())
def test_oracle_lifting_sums_replay_the_reference_trajectory(name):
    spec, initial, charges, events, final = load_trajectory(name)
    chain = oracle.Chain(oracle_system(spec), initial, charges)
    chain.run(len(events), record=False)
    assert chain.liftings() == replay_liftings(spec, initial, events)


def test_estimator_functions_on_known_configurations():
    length = 10.0
    # two units 1.5 apart across the boundary: minimum image distance 1.5
    pair = np.array([[0.25, 5.0, 5.0], [8.75, 5.0, 5.0]])
    assert np.allclose(estimators.pair_distances(pair, length), [1.5])
    expected = (1.0 / 1.5) ** 12 - (1.0 / 1.5) ** 6
    assert estimators.lennard_jones_energy(pair, length) == pytest.approx(expected, rel=1e-14)
    assert estimators.pair_histogram(pair, length, 10, 5.0).tolist() == [0, 0, 0, 1, 0, 0, 0, 0, 0, 0]
    # an ideal gas has g(r) = 1 within its noise
    rng = np.random.default_rng(0)
    counts = sum(estimators.pair_histogram(rng.uniform(0, length, (200, 3)), length, 10, 5.0) for _ in range(50))
    r, g = estimators.pair_correlation(counts, 50, 200, length, 5.0)
    assert np.all(np.abs(g[2:] - 1.0) < 0.05)
    assert estimators.pressure(3.0, 2.0) == 2.5
    assert estimators.ratio_of_sums([1.0, 3.0], [2.0, 2.0])[0] == 1.0


def oracle_samples(spec, chains, samples, seed):
    """Per-chain samples of `chains` independent oracle chains from the fixture's initial state."""
    from tests.golden.make_reference_trajectories import initial_state
    length, initial, _ = initial_state(spec)
    system_spec = dict(spec, rng_key=0)

    def one(c):
        system = oracle_system(dict(system_spec, rng_key=oracle.chain_key(seed, c)))
        chain = oracle.Chain(system, initial)
        t = 0
        for t in range(1, spec["burn_in"] + 1):
            chain.run(10 ** 7, stop_time=t * spec["chain_time"], record=False)
        energy, lift, hist = [], [], np.zeros(spec["bins"], dtype=np.int64)
        previous = chain.liftings()[0]
        for k in range(t + 1, t + samples + 1):
            chain.run(10 ** 7, stop_time=k * spec["chain_time"], record=False)
            config = chain.positions()
            energy.append(estimators.lennard_jones_energy(config, length)
                          if spec["potential"] == "lennard_jones" else 0.0)
            total = chain.liftings()[0]
            lift.append(total - previous)
            previous = total
            hist += estimators.pair_histogram(config, length, spec["bins"], spec["r_max"])
        return energy, lift, hist

    with concurrent.futures.ThreadPoolExecutor(max_workers=8) as pool:
        results = list(pool.map(one, range(chains)))
    return [r[0] for r in results], [r[1] for r in results], [r[2] for r in results]


@pytest.mark.parametrize("name", estimator_names())
def test_oracle_long_runs_reproduce_the_reference_estimators(name):
    spec, reference = reference_estimates(name)
    energies, lifts, histograms = oracle_samples(spec, chains=16, samples=spec["samples"], seed=77)
    other = sampled_estimates(spec, energies, lifts, histograms)
    assert compare(reference, other) == []
