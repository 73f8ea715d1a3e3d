"""Generate ``composite_events.json``: events of two composite objects recorded from reference runs.

Run in a container that holds the JeLLyFysh source tree with its cffi extensions built:

    python tests/golden/make_composite_golden.py /path/to/jellyfysh/tree

The reference runs unchanged (Python's ``random``, seeded) from its own configuration files for dipoles (two point
charges per composite object, the three lifting schemes) and water (three per composite object, inside-first
lifting); output files go to a scratch directory.  Every call of ``TwoCompositeObjectSummedBoundingPotentialEventHandler``
(``event_handler/two_composite_object_summed_bounding_potential_event_handler.py:119-202``) is observed:

* ``send_event_time``: the active unit (position, charge, velocity) and the target composite object's units before
  the time slice, the potential change drawn for each target unit (``random.expovariate``) and the displacement the
  bounding potential returned for each; the candidate displacement is their minimum;
* ``send_out_state``: the units of both composite objects at the event (time-sliced), sorted by identifier as the
  handler sorts them, the active unit's index, whether the local composite object comes first, every
  ``random.uniform`` call (arguments and value: the thinning draw, then the lifting draws) and the outcome (rejected,
  or the unit that became active).
"""
import configparser
import json
import os
import random
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
CONFIGS = {
    "dipoles_inside_first": ("2018_JCP_149_064113/dipoles/dipole_factors_inside_first.ini", 11),
    "dipoles_outside_first": ("2018_JCP_149_064113/dipoles/dipole_factors_outside_first.ini", 12),
    "dipoles_ratio": ("2018_JCP_149_064113/dipoles/dipole_factors_ratio.ini", 13),
    "water_inside_first": ("2018_JCP_149_064113/water/coulomb_power_bounded_lj_cell_bounded.ini", 14),
}
ACCEPTED = 40   # recorded accepted out-states per configuration
REJECTED = 20   # recorded rejected (thinned) out-states per configuration
TIMES = 80      # recorded event-time calls per configuration


class Stop(Exception):
    pass


def run_one(tree, name, out):
    path, seed = CONFIGS[name]
    os.chdir(os.path.join(tree, "jellyfysh"))
    sys.path.insert(0, tree)
    import logging
    logging.disable(logging.ERROR)
    from jellyfysh.base import factory
    from jellyfysh.base.strings import to_camel_case
    from jellyfysh.event_handler import two_composite_object_summed_bounding_potential_event_handler as module
    handler_class = module.TwoCompositeObjectSummedBoundingPotentialEventHandler

    config = configparser.ConfigParser()
    config.read(os.path.join("config_files", path))
    scratch = tempfile.mkdtemp()
    for section in config.sections():
        if config.has_option(section, "filename") and section != "FactorTypeMaps":
            config.set(section, "filename", os.path.join(scratch, section + ".dat"))
    setting_section = config["HypercubicSetting"]
    record = {"config": path, "system_length": float(setting_section["system_length"]),
              "beta": float(setting_section["beta"]), "times": [], "out_states": []}
    for section in config.sections():
        if config.has_option(section, "bounding_potential") and config.has_option(section, "lifting"):
            handler_section = section
    record["lifting"] = config.get(handler_section, "lifting").strip()
    record["charge"] = config.get(handler_section, "charge").strip()

    ctx = {"calls": None}
    original_expovariate, original_uniform = random.expovariate, random.uniform

    def expovariate(lambd):
        value = original_expovariate(lambd)
        if ctx["calls"] is not None:
            ctx["calls"].append(("expovariate", [lambd], value))
        return value

    def uniform(a, b):
        value = original_uniform(a, b)
        if ctx["calls"] is not None:
            ctx["calls"].append(("uniform", [a, b], value))
        return value
    random.expovariate, random.uniform = expovariate, uniform

    charge = record["charge"]

    def unit_record(unit):
        return {"position": list(unit.position), "charge": unit.charge[charge]}

    original_slice = handler_class._time_slice_all_units_in_state
    original_time = handler_class.send_event_time
    original_out = handler_class.send_out_state

    def time_slice(self):
        # called at the end of send_event_time: positions are those before the slice
        if ctx.get("time") is not None:
            ctx["time"].update(active=unit_record(self._active_leaf_unit),
                               velocity=list(self._active_leaf_unit.velocity),
                               targets=[unit_record(u) for u in self._target_leaf_units])
        return original_slice(self)

    bound_calls = []

    def send_event_time(self, in_state):
        if "coulomb" not in record:  # the parameters the reference's potentials were built with
            potential, bound = self._potential, self._bounding_potential
            record["potential"] = type(potential).__name__
            record["bounding_potential"] = type(bound).__name__
            record["lifting_class"] = type(self._lifting).__name__
            record["coulomb"] = {"alpha": potential._alpha, "fourier_cutoff": potential._fourier_cutoff,
                                 "position_cutoff": potential._position_cutoff, "prefactor": potential._prefactor}
            record["bound"] = {"prefactor": bound._prefactor}
        ctx["time"] = {}
        ctx["calls"] = []
        original_displacement = self._bounding_potential.displacement
        del bound_calls[:]

        def displacement(*args):
            value = original_displacement(*args)
            bound_calls.append(value)
            return value
        self._bounding_potential.displacement = displacement
        try:
            result = original_time(self, in_state)
        finally:
            self._bounding_potential.displacement = original_displacement
        entry = ctx["time"]
        entry["potential_changes"] = [value for kind, _, value in ctx["calls"] if kind == "expovariate"]
        entry["displacements"] = list(bound_calls)
        ctx["time"] = None
        ctx["calls"] = None
        if len(record["times"]) < TIMES:
            record["times"].append(entry)
        return result

    def send_out_state(self):
        local = self._local_leaf_units
        target = self._target_leaf_units
        entry = {"velocity": list(self._active_leaf_unit.velocity),
                 "local": [unit_record(u) for u in local], "target": [unit_record(u) for u in target],
                 "active_index": [i for i, u in enumerate(local) if u is self._active_leaf_unit][0],
                 "local_first": local[0].identifier[0] < target[0].identifier[0]}
        units = list(local) + list(target)
        ctx["calls"] = []
        try:
            result = original_out(self)
        finally:
            calls, ctx["calls"] = ctx["calls"], None
        entry["uniform_calls"] = [[args, value] for kind, args, value in calls if kind == "uniform"]
        moved = [i for i, u in enumerate(units) if u.velocity is not None]
        assert len(moved) == 1
        entry["accepted"] = len(entry["uniform_calls"]) > 1
        entry["new_active"] = moved[0] if entry["accepted"] else -1
        kept = sum(1 for e in record["out_states"] if e["accepted"] == entry["accepted"])
        if kept < (ACCEPTED if entry["accepted"] else REJECTED):
            record["out_states"].append(entry)
        if len(record["out_states"]) >= ACCEPTED + REJECTED and len(record["times"]) >= TIMES:
            raise Stop()
        return result

    handler_class._time_slice_all_units_in_state = time_slice
    handler_class.send_event_time = send_event_time
    handler_class.send_out_state = send_out_state

    random.seed(seed)
    factory.build_from_config(config, to_camel_case(config.get("Run", "setting")), "jellyfysh.setting")
    mediator = factory.build_from_config(config, to_camel_case(config.get("Run", "mediator")), "jellyfysh.mediator")
    try:
        mediator.run()
    except Stop:
        pass
    with open(out, "w") as handle:
        json.dump(record, handle)


def main(tree):
    records = {}
    with tempfile.TemporaryDirectory() as scratch:
        for name in CONFIGS:
            out = os.path.join(scratch, name + ".json")
            subprocess.run([sys.executable, os.path.abspath(__file__), "--one", tree, name, out], check=True)
            with open(out) as handle:
                records[name] = json.load(handle)
            print("%s: %d event times, %d out-states (%d accepted)" % (
                name, len(records[name]["times"]), len(records[name]["out_states"]),
                sum(e["accepted"] for e in records[name]["out_states"])))
    path = os.path.join(HERE, "composite_events.json")
    with open(path, "w") as handle:
        json.dump({"source": "reference runs of its dipole and water configurations", "systems": records}, handle)
        handle.write("\n")
    print("wrote", path)


if __name__ == "__main__":
    from _tree import tree_argument
    if len(sys.argv) > 1 and sys.argv[1] == "--one":
        run_one(sys.argv[2], sys.argv[3], sys.argv[4])
    else:
        main(tree_argument(sys.argv))
