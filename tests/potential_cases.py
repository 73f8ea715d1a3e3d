"""Map the reference's potential known-answer cases onto plain parameter records.

Each case of ``golden/potential_known_answers.json`` holds the reference call (potential class, constructor
arguments, method, velocity, separation, charges, potential change), the value the reference returned and the
known answer of the reference test.  ``normalise`` turns it into a dict with 3D vectors (2D hard-disk cases are
padded with a zero component, which leaves every sum unchanged).
"""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def load_cases():
    with open(os.path.join(HERE, "golden", "potential_known_answers.json")) as handle:
        return json.load(handle)["cases"]


def _pad(vector):
    vector = [float(v) for v in vector]
    return vector + [0.0] * (3 - len(vector))


def normalise(case):
    params = dict(case["params"])
    positional = params.pop("_args", [])
    attributes = case.get("attributes", {})
    args = list(case["args"])
    kwargs = dict(case["kwargs"])
    record = dict(potential=case["potential"], method=case["method"], reference=case["reference"],
                  expected=case["expected"], places=case["places"], system_length=case["system_length"],
                  test=case["test"], meets_known_answer=case.get("reference_meets_known_answer", True))
    record["velocity"] = _pad(args[0])
    record["separation"] = _pad(args[1])
    rest = args[2:]
    if "potential_change" in kwargs:
        rest = rest + [kwargs["potential_change"]]
    name = case["potential"]
    if name == "HardSpherePotential":
        record["radius"] = float(positional[0] if positional else params["radius"])
    elif name == "InversePowerPotential":
        record["power"] = float(attributes.get("_power", params["power"]))
        record["prefactor"] = float(attributes.get("_prefactor", params["prefactor"]))
    elif name == "LennardJonesPotential":
        record["prefactor"] = float(attributes.get("_prefactor", params.get("prefactor", 1.0)))
        record["sigma"] = float(attributes.get("_characteristic_length", params.get("characteristic_length", 1.0)))
    elif name == "DisplacedEvenPowerPotential":
        record["r0"] = float(attributes.get("_equilibrium_separation", params["equilibrium_separation"]))
        record["power"] = int(attributes.get("_power", params["power"]))
        record["prefactor"] = float(attributes.get("_prefactor", params.get("prefactor", 1.0)))
    elif name == "InversePowerCoulombBoundingPotential":
        record["prefactor"] = float(attributes.get("_prefactor", params.get("prefactor", 1.5837)))
    elif name == "MergedImageCoulombPotential":
        record["alpha"] = float(attributes.get("_alpha", params.get("alpha", 3.45)))
        record["fourier_cutoff"] = int(attributes.get("_fourier_cutoff", params.get("fourier_cutoff", 6)))
        record["position_cutoff"] = int(attributes.get("_position_cutoff", params.get("position_cutoff", 2)))
        record["prefactor"] = float(attributes.get("_prefactor", params.get("prefactor", 1.0)))
    charged = name in ("InversePowerPotential", "InversePowerCoulombBoundingPotential", "MergedImageCoulombPotential")
    if charged:
        record["charges"] = (float(rest[0]), float(rest[1]))
        rest = rest[2:]
    else:
        record["charges"] = (1.0, 1.0)
    record["potential_change"] = float(rest[0]) if (case["method"] == "displacement" and rest) else 0.0
    return record


def places_ok(value, expected, places):
    if value == expected:
        return True
    return round(abs(value - expected), places if places is not None else 7) == 0
