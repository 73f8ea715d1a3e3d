"""The oracle against the reference's potential known-answer tests (CPU only).

Each case was recorded from the reference's own ``unittests/test_potential`` run: the oracle must return the
reference's value bit for bit and meet the test's known answer to the test's number of places.
"""
import math

import pytest

import oracle
from tests.potential_cases import load_cases, normalise, places_ok

CASES = [normalise(case) for case in load_cases()]


def oracle_value(c):
    v, s = c["velocity"], c["separation"]
    name, method = c["potential"], c["method"]
    if name == "HardSpherePotential":
        return oracle.hs_displacement(c["radius"], v, s)
    if name == "InversePowerPotential":
        if method == "displacement":
            return oracle.ip_displacement(c["power"], c["prefactor"], v, s, *c["charges"], c["potential_change"])
        return oracle.ip_derivative(c["power"], c["prefactor"], v, s, *c["charges"])
    if name == "LennardJonesPotential":
        if method == "displacement":
            return oracle.lj_displacement(c["prefactor"], c["sigma"], v, s, c["potential_change"])
        return oracle.lj_derivative(c["prefactor"], c["sigma"], v, s)
    if name == "DisplacedEvenPowerPotential":
        if method == "displacement":
            return oracle.dep_displacement(c["r0"], c["power"], c["prefactor"], v, s, c["potential_change"])
        return oracle.dep_derivative(c["r0"], c["power"], c["prefactor"], v, s)
    if name == "InversePowerCoulombBoundingPotential":
        if method == "displacement":
            return oracle.ipcb_displacement(c["prefactor"], c["system_length"], v, s, *c["charges"],
                                            c["potential_change"])
        return oracle.ipcb_derivative(c["prefactor"], v, s, *c["charges"])
    if name == "MergedImageCoulombPotential":
        return oracle.mic_derivative(c["alpha"], c["fourier_cutoff"], c["position_cutoff"], c["prefactor"],
                                     c["system_length"], v, s, *c["charges"])
    raise KeyError(name)


@pytest.mark.parametrize("case", CASES, ids=[c["test"].split(".")[-1] + ":" + c["method"] for c in CASES])
def test_oracle_matches_reference_bitwise(case):
    value = oracle_value(case)
    reference = case["reference"]
    if math.isinf(reference):
        assert value == reference
    else:
        assert value == reference, (value, reference, value - reference)
    if case["meets_known_answer"]:
        assert places_ok(value, case["expected"], case["places"])


def test_every_potential_is_covered():
    names = {(c["potential"], c["method"]) for c in CASES}
    for name in ("HardSpherePotential", "InversePowerPotential", "LennardJonesPotential",
                 "DisplacedEvenPowerPotential", "InversePowerCoulombBoundingPotential"):
        assert (name, "displacement") in names
    assert ("MergedImageCoulombPotential", "derivative") in names
