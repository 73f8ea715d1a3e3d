"""Molecular cell-bounding and cell-veto events recorded from reference runs (``golden/composite_cell_events.json``,
written by ``golden/make_composite_cell_golden.py``), flattened to the arrays of the batched entry points."""
import json
import os

import numpy as np

from tests.composite_cases import out_state_arrays

HERE = os.path.dirname(os.path.abspath(__file__))
SCHEMES = {"InsideFirstLifting": "inside_first", "OutsideFirstLifting": "outside_first", "RatioLifting": "ratio"}


def load_cell_systems():
    with open(os.path.join(HERE, "golden", "composite_cell_events.json")) as handle:
        return json.load(handle)["systems"]


def model_of(record):
    """The model of a recorded system: units per object, the merged-image Coulomb parameters, the lifting scheme."""
    coulomb = record["coulomb"]
    return {"units": len(record["out_states"][0]["local"]), "alpha": float(coulomb["alpha"]),
            "fourier_cutoff": int(coulomb["fourier_cutoff"]), "position_cutoff": int(coulomb["position_cutoff"]),
            "coulomb_prefactor": float(coulomb["prefactor"]), "system_length": float(record["system_length"]),
            "scheme": SCHEMES[record["lifting_class"]]}


def bound_tables(record):
    """upper, lower [cells][3] with NaN rows for the nearby cells; the Walker totals by direction (cell veto)."""
    tables = record["tables"]
    nan = [float("nan")] * 3
    upper = np.array([row if row is not None else nan for row in tables["upper"]], dtype=np.float64)
    lower = np.array([row if row is not None else nan for row in tables["lower"]], dtype=np.float64)
    return upper, lower, tables.get("walker_upper"), tables.get("walker_lower")


def time_arrays(record):
    times = record["times"]
    out = {"relative_cell": np.array([t["relative_cell"] for t in times], dtype=np.int32),
           "velocity": np.array([[t["speed"] if d == t["direction"] else 0.0 for d in range(3)] for t in times],
                                dtype=np.float64),
           "potential_change": np.array([t["potential_change"] for t in times], dtype=np.float64),
           "rate": np.array([t["bounding_event_rate"] for t in times], dtype=np.float64),
           "time_stamp": np.array([t["time_stamp"] for t in times], dtype=np.float64),
           "event_time": np.array([t["event_time"] for t in times], dtype=np.float64)}
    if record["kind"] == "cell_bounding":
        out["active_charge"] = np.array([t["active_charge"] for t in times], dtype=np.float64)
        out["target_charges"] = np.array([t["target_charges"] for t in times], dtype=np.float64)
    else:
        # the cell veto's charge factor is the active charge
        out["active_charge"] = np.array([t["charge_factor"] for t in times], dtype=np.float64)
        out["walker_total"] = np.array([t["walker_total_rate"] for t in times], dtype=np.float64)
    return out


def out_arrays(record):
    """The recorded out-states with a target, as for the summed handler, plus the bounding event rate the thinning
    drew against."""
    out = out_state_arrays(record)
    out["given_rate"] = np.array([e["bounding_event_rate"] for e in record["out_states"]], dtype=np.float64)
    return out


def walkers(record):
    """The cell veto's Walker tables: {(which, direction): {"items", "rates", "table", "mean_rate", "total_rate"}}
    with which 0 for the upper bounds and 1 for the lower ones."""
    tables = record["tables"]["walkers"]
    return {(which, d): w for which, name in enumerate(("upper", "lower")) for d, w in enumerate(tables[name])}


def walker_draws(record):
    """Per recorded cell-veto event time: (which, direction, table index of random.choice, random.uniform value,
    sampled relative cell)."""
    return [(0 if t["charge_factor"] > 0.0 else 1, t["direction"], t["walker_choice"], t["walker_uniform"],
             t["relative_cell"]) for t in record["times"]]
