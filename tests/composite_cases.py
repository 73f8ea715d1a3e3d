"""Events of two composite objects recorded from reference runs (``golden/composite_events.json``, written by
``golden/make_composite_golden.py``), flattened to the arrays of the batched entry points."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SCHEMES = {"inside_first_lifting": "inside_first", "outside_first_lifting": "outside_first",
           "ratio_lifting": "ratio"}


def load_systems():
    with open(os.path.join(HERE, "golden", "composite_events.json")) as handle:
        return json.load(handle)["systems"]


def model_of(record):
    """The model of a recorded system: units per object, the potentials' parameters and the lifting scheme."""
    coulomb = record["coulomb"]
    units = len(record["times"][0]["targets"])
    return {"units": units, "alpha": float(coulomb["alpha"]), "fourier_cutoff": int(coulomb["fourier_cutoff"]),
            "position_cutoff": int(coulomb["position_cutoff"]), "coulomb_prefactor": float(coulomb["prefactor"]),
            "bound_prefactor": float(record["bound"]["prefactor"]), "system_length": float(record["system_length"]),
            "scheme": SCHEMES[record["lifting"]]}


def time_arrays(record):
    times = record["times"]
    return {"velocity": np.array([t["velocity"] for t in times], dtype=np.float64),
            "active_position": np.array([t["active"]["position"] for t in times], dtype=np.float64),
            "active_charge": np.array([t["active"]["charge"] for t in times], dtype=np.float64),
            "target_positions": np.array([[u["position"] for u in t["targets"]] for t in times], dtype=np.float64),
            "target_charges": np.array([[u["charge"] for u in t["targets"]] for t in times], dtype=np.float64),
            "potential_changes": np.array([t["potential_changes"] for t in times], dtype=np.float64),
            "expected": np.array([min(t["displacements"]) for t in times], dtype=np.float64)}


def out_state_arrays(record):
    """Arrays of the recorded out-states; draws are the values the reference's random.uniform returned (the ratio
    scheme's third draw is its get_active_identifier draw; a thinned event has one draw)."""
    outs = record["out_states"]
    draws = np.zeros((len(outs), 3), dtype=np.float64)
    for i, e in enumerate(outs):
        for k, (_, value) in enumerate(e["uniform_calls"][:3]):
            draws[i, k] = value
    return {"velocity": np.array([e["velocity"] for e in outs], dtype=np.float64),
            "local_positions": np.array([[u["position"] for u in e["local"]] for e in outs], dtype=np.float64),
            "local_charges": np.array([[u["charge"] for u in e["local"]] for e in outs], dtype=np.float64),
            "active_index": np.array([e["active_index"] for e in outs], dtype=np.int32),
            "target_positions": np.array([[u["position"] for u in e["target"]] for e in outs], dtype=np.float64),
            "target_charges": np.array([[u["charge"] for u in e["target"]] for e in outs], dtype=np.float64),
            "local_first": np.array([1 if e["local_first"] else 0 for e in outs], dtype=np.int32),
            "draws": draws,
            "new_active": np.array([e["new_active"] for e in outs], dtype=np.int32),
            # the reference's random.uniform bounds: the summed bounding rate, then the event rate (lifting insert)
            "bounding_rate": np.array([e["uniform_calls"][0][0][1] for e in outs], dtype=np.float64),
            "event_rate": np.array([e["uniform_calls"][1][0][1] if e["accepted"] else np.nan for e in outs],
                                   dtype=np.float64)}
