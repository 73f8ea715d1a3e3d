"""Estimators of long ECMC runs: pressure, mean potential energy and pair correlation.

The reference writes raw samples (pair separations, ``separation_output_handler.py:75-97``) and leaves the
estimators to its analysis scripts; it has no pressure or energy estimator.  These functions compute the three
estimators from the same kind of samples whichever path produced them (the GPU engine's device observations,
the oracle's states, or positions sampled from the reference's own event loop), so that long runs of the paths
can be compared within their statistical errors:

* pressure from the liftings (event-chain virial): beta P / rho = 1 + <sum over liftings of the separation
  target - active along the direction of motion> / (chain displacement);
* mean potential energy per unit of configurations sampled at fixed times (the end of every chain);
* pair correlation g(r) from the histogram of minimum-image pair distances.

Errors are standard errors over independent blocks (independent chains, or batches of consecutive samples).
"""
from typing import Optional, Sequence, Tuple

import numpy as np


def minimum_image(separations: np.ndarray, length: float) -> np.ndarray:
    """((s + L/2) % L) - L/2 componentwise (HypercubicPeriodicBoundaries.separation_vector)."""
    return np.mod(separations + 0.5 * length, length) - 0.5 * length


def pair_distances(positions: np.ndarray, length: float) -> np.ndarray:
    """Minimum-image distances of all unordered pairs of one configuration [n, 3]."""
    i, j = np.triu_indices(len(positions), k=1)
    s = minimum_image(positions[j] - positions[i], length)
    return np.sqrt(np.einsum("ij,ij->i", s, s))


def lennard_jones_energy(positions: np.ndarray, length: float, prefactor: float = 1.0, sigma: float = 1.0) -> float:
    """Potential energy sum_pairs k ((sigma/r)^12 - (sigma/r)^6), the reference's LennardJonesPotential
    (lennard_jones_potential.py:83-98, k = its prefactor) with minimum-image separations and no cutoff."""
    r = pair_distances(positions, length)
    x6 = (sigma / r) ** 6
    return float(np.sum(prefactor * (x6 * x6 - x6)))


def pair_histogram(positions: np.ndarray, length: float, bins: int, r_max: float) -> np.ndarray:
    """Counts of the pair distances of one configuration in [0, r_max) with `bins` equal bins."""
    r = pair_distances(positions, length)
    counts, _ = np.histogram(r[r < r_max], bins=bins, range=(0.0, r_max))
    return counts.astype(np.int64)


def pair_correlation(counts: np.ndarray, samples: int, n: int, length: float, r_max: float) -> Tuple[np.ndarray,
                                                                                                     np.ndarray]:
    """g(r) at the bin centres from summed pair-distance counts of `samples` configurations of n units."""
    counts = np.asarray(counts, dtype=np.float64)
    bins = counts.shape[-1]
    edges = np.linspace(0.0, r_max, bins + 1)
    shell = 4.0 / 3.0 * np.pi * (edges[1:] ** 3 - edges[:-1] ** 3)
    ideal = samples * 0.5 * n * (n - 1) * shell / length ** 3
    return 0.5 * (edges[1:] + edges[:-1]), counts / ideal


def pressure(lift_sum: float, displacement: float) -> float:
    """beta P / rho = 1 + (excess displacement of the liftings) / (displacement of the chains)."""
    return 1.0 + lift_sum / displacement


def block_mean(values: Sequence[float], blocks: Optional[int] = None) -> Tuple[float, float]:
    """Mean and standard error of the mean over `blocks` consecutive blocks (each value its own block if None)."""
    v = np.asarray(values, dtype=np.float64)
    if blocks is not None:
        usable = (len(v) // blocks) * blocks
        v = v[:usable].reshape(blocks, -1).mean(axis=1)
    if len(v) < 2:
        return float(v.mean()), float("inf")
    return float(v.mean()), float(v.std(ddof=1) / np.sqrt(len(v)))


def ratio_of_sums(numerators: Sequence[float], denominators: Sequence[float]) -> Tuple[float, float]:
    """sum(x) / sum(y) over independent blocks with its delta-method standard error."""
    x = np.asarray(numerators, dtype=np.float64)
    y = np.asarray(denominators, dtype=np.float64)
    k = len(x)
    ratio = x.sum() / y.sum()
    if k < 2:
        return float(ratio), float("inf")
    residual = x - ratio * y
    error = np.sqrt(k / (k - 1.0) * np.sum(residual ** 2)) / y.sum()
    return float(ratio), float(error)


def within(a: Tuple[float, float], b: Tuple[float, float], sigmas: float = 3.0) -> bool:
    """|a - b| <= sigmas * sqrt(err_a^2 + err_b^2) for (mean, error) pairs."""
    return abs(a[0] - b[0]) <= sigmas * float(np.hypot(a[1], b[1]))


def chi_square(a: np.ndarray, a_err: np.ndarray, b: np.ndarray, b_err: np.ndarray) -> Tuple[float, int]:
    """Chi-square of two binned estimates with independent errors (bins with no error on either side skipped)."""
    variance = np.asarray(a_err, dtype=np.float64) ** 2 + np.asarray(b_err, dtype=np.float64) ** 2
    use = variance > 0
    chi2 = float(np.sum((np.asarray(a)[use] - np.asarray(b)[use]) ** 2 / variance[use]))
    return chi2, int(use.sum())


def chi_square_within(chi2: float, dof: int, sigmas: float = 3.0) -> bool:
    """chi2 below its mean plus `sigmas` standard deviations (dof + sigmas sqrt(2 dof))."""
    return chi2 <= dof + sigmas * np.sqrt(2.0 * dof)
