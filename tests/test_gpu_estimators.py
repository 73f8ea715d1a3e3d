"""Estimators of long runs on the GPU engine.

* The lifting sums of the engine (exact and mixed precision) equal the oracle's on the reference trajectories
  (bit for bit for hard spheres, to 1e-12 of the box per lifting otherwise), and so the sums replayed from the
  reference's own events.
* The device observables (potential energy, pair-distance histogram) agree with the host estimator functions on
  the same configurations (FP32 pair terms: energy to 1e-5 relative, histograms up to pairs on bin edges).
* Long runs of many chains in mixed precision reproduce the reference's estimators (``golden/estimators_*.npz``,
  the reference's event loop with its own random numbers): energy and pressure within 3 standard errors, the
  pair correlation by a chi-square within 3 standard deviations.
"""
import numpy as np
import pytest

import oracle
from jellyfysh_gb300 import estimators
from tests.estimator_cases import compare, estimator_names, reference_estimates, sampled_estimates
from tests.trajectory_cases import load_trajectory, oracle_system, trajectory_names

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def chain_spec(spec, rng_key):
    from jellyfysh_gb300 import ChainSpec
    return ChainSpec(n=spec["n"], system_length=spec["system_length"], cells_per_side=spec["cells_per_side"],
                     potential=spec["potential"], far=spec["far"], neighbor_layers=spec["neighbor_layers"],
                     max_occupants=1, beta=spec["beta"], chain_time=spec["chain_time"], speed=1.0,
                     hs_radius=spec.get("radius", 0.0), estimator_points=spec.get("estimator_points", 10),
                     estimator_prefactor=spec.get("estimator_prefactor", 1.5), rng_key=rng_key)


@pytest.mark.parametrize("mode", ["exact", "mixed"])
@pytest.mark.parametrize("name", trajectory_names())
def test_lifting_sums_equal_the_oracle(name, mode):
    from jellyfysh_gb300 import ChainBatch
    spec, initial, charges, events, final = load_trajectory(name)
    batch = ChainBatch([chain_spec(spec, spec["rng_key"])], [initial], None if charges is None else [charges])
    batch.run(len(events), mode=mode)
    batch.check_status()
    state = batch.state()[0]
    chain = oracle.Chain(oracle_system(spec), initial, charges)
    chain.run(len(events), record=False)
    lift_sum, liftings = chain.liftings()
    assert int(state["liftings"]) == liftings
    if spec["potential"] == "hard_sphere":
        assert float(state["lift_sum"]) == lift_sum  # positions bit for bit (square roots only)
    else:
        # positions agree to 1e-12 of the box (correctly rounded powers, CUDA's transcendentals)
        assert float(state["lift_sum"]) == pytest.approx(lift_sum, abs=1e-12 * spec["system_length"] * liftings)
    batch.close()


def test_device_observables_match_the_host_estimators():
    from jellyfysh_gb300 import ChainBatch
    spec, initial, charges, events, final = load_trajectory("lennard_jones_n128_two_layers_cell_veto")
    chains = 8
    batch = ChainBatch([chain_spec(spec, None)] * chains, [initial] * chains, seed=5)
    batch.run(300, mode="mixed")
    batch.check_status()
    length = spec["system_length"]
    bins, r_max = 50, 0.5 * length
    energy, histogram = batch.observe(bins, r_max)
    energy = energy.cpu().numpy()
    histogram = histogram.cpu().numpy()
    for c in range(chains):
        config = batch.positions(c)
        assert energy[c] == pytest.approx(estimators.lennard_jones_energy(config, length), rel=1e-5)
        expected = estimators.pair_histogram(config, length, bins, r_max)
        assert abs(int(histogram[c].sum()) - int(expected.sum())) <= 2
        assert np.abs(histogram[c] - expected).sum() <= 4
    # the histogram accumulates over calls
    _, twice = batch.observe(bins, r_max, histogram=torch.tensor(histogram, device=batch.device))
    assert np.array_equal(twice.cpu().numpy(), 2 * histogram)
    batch.close()


def gpu_samples(spec, chains, samples, seed, max_events):
    """Per-chain samples of independent GPU chains (mixed precision) from the fixture's initial state."""
    from jellyfysh_gb300 import ChainBatch
    from tests.golden.make_reference_trajectories import initial_state
    length, initial, _ = initial_state(spec)
    batch = ChainBatch([chain_spec(spec, None)] * chains, [initial] * chains, seed=seed)
    t = 0
    for t in range(1, spec["burn_in"] + 1):
        batch.run(max_events, stop_time=t * spec["chain_time"], mode="mixed")
    histogram = torch.zeros((chains, spec["bins"]), dtype=torch.int64, device=batch.device)
    energies, lifts = [], []
    previous = batch.state()["lift_sum"].copy()
    for k in range(t + 1, t + samples + 1):
        batch.run(max_events, stop_time=k * spec["chain_time"], mode="mixed")
        state = batch.state()
        assert (state["stopped"] == 1).all(), "raise max_events: a chain did not reach the sampling time"
        energy, histogram = batch.observe(spec["bins"], spec["r_max"], histogram=histogram)
        energies.append(energy.cpu().numpy() if spec["potential"] == "lennard_jones" else np.zeros(chains))
        lifts.append(state["lift_sum"] - previous)
        previous = state["lift_sum"].copy()
    batch.check_status()
    batch.close()
    return np.array(energies).T, np.array(lifts).T, histogram.cpu().numpy()


@pytest.mark.parametrize("name", estimator_names())
def test_long_gpu_runs_reproduce_the_reference_estimators(name):
    spec, reference = reference_estimates(name)
    max_events = 600 if spec["potential"] == "lennard_jones" else 200
    energies, lifts, histograms = gpu_samples(spec, chains=256, samples=spec["samples"] // 4, seed=31,
                                              max_events=max_events)
    other = sampled_estimates(spec, energies, lifts, histograms)
    assert compare(reference, other) == []
