"""Long-run estimators of the reference fixtures (``golden/estimators_*.npz``) and of chains run by other paths.

``reference_estimates`` turns the samples recorded from the reference's own event loop into (mean, error) pairs;
``sampled_estimates`` does the same for per-chain samples of the oracle or the GPU engine, so that every path
goes through the same estimator code (``jellyfysh_gb300.estimators``).
"""
import glob
import json
import os

import numpy as np

from jellyfysh_gb300 import estimators

HERE = os.path.dirname(os.path.abspath(__file__))


def estimator_names():
    return sorted(os.path.basename(p)[len("estimators_"):-len(".npz")]
                  for p in glob.glob(os.path.join(HERE, "golden", "estimators_*.npz")))


def load_fixture(name):
    data = np.load(os.path.join(HERE, "golden", "estimators_%s.npz" % name))
    spec = json.loads(str(data["spec"]))
    return spec, data


def _estimates(spec, energy_blocks, lift_blocks, displacement_blocks, histogram_blocks, samples_per_block):
    """(mean, error) of energy per unit and beta P / rho, and g(r) with its per-bin errors, from blocks."""
    n = spec["n"]
    energy = estimators.block_mean(np.asarray(energy_blocks) / n)
    ratio, ratio_error = estimators.ratio_of_sums(lift_blocks, displacement_blocks)
    g_blocks = np.array([estimators.pair_correlation(h, s, n, spec["system_length"], spec["r_max"])[1]
                         for h, s in zip(histogram_blocks, samples_per_block)])
    g_mean = g_blocks.mean(axis=0)
    g_error = g_blocks.std(axis=0, ddof=1) / np.sqrt(len(g_blocks))
    return {"energy": energy, "pressure": (1.0 + ratio, ratio_error), "g": (g_mean, g_error)}


def reference_estimates(name):
    """Estimates of the reference's independent runs (each run one block)."""
    spec, data = load_fixture(name)
    return spec, sampled_estimates(spec, data["energy"], data["lift"], data["histograms"])


def sampled_estimates(spec, energies, lifts, histograms):
    """Estimates of independent chains or runs (each one block): energies [chains][samples], lifts
    [chains][samples] (lifting sums per chain segment), histograms [chains][bins] (summed over the samples)."""
    energies = np.asarray(energies, dtype=np.float64)
    lifts = np.asarray(lifts, dtype=np.float64)
    samples = energies.shape[1]
    displacement = np.full(len(energies), samples * spec["chain_time"] * spec["speed"])
    return _estimates(spec, energies.mean(axis=1), lifts.sum(axis=1), displacement, histograms,
                      [samples] * len(energies))


def compare(reference, other, sigmas=3.0):
    """Failures of `other` against `reference`: energy and pressure within `sigmas` standard errors, g(r) by a
    chi-square within `sigmas` standard deviations of its distribution."""
    failures = []
    for key in ("energy", "pressure"):
        if not estimators.within(reference[key], other[key], sigmas):
            failures.append("%s: reference %.6g +- %.2g, other %.6g +- %.2g" % (key, reference[key][0],
                                                                               reference[key][1], other[key][0],
                                                                               other[key][1]))
    # bins the reference populates (g > 0.05): the Gaussian errors of nearly empty bins mean little
    use = reference["g"][0] > 0.05
    chi2, dof = estimators.chi_square(reference["g"][0][use], reference["g"][1][use], other["g"][0][use],
                                      other["g"][1][use])
    if not estimators.chi_square_within(chi2, dof, sigmas):
        failures.append("g(r): chi2 %.1f for %d bins" % (chi2, dof))
    return failures
