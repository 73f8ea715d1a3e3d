"""Generate ``composite_cell_events.json``: molecular cell-bounding and cell-veto events recorded from reference runs.

Run in a container that holds the JeLLyFysh source tree with its cffi extensions built:

    python tests/golden/make_composite_cell_golden.py /path/to/jellyfysh/tree

The reference runs unchanged (Python's ``random``, seeded) from its own configuration files: dipoles with the
molecular cell-bounding potential (``TwoCompositeObjectCellBoundingPotentialEventHandler``,
``event_handler/two_composite_object_cell_bounding_potential_event_handler.py:153-265``), dipoles and water with the
molecular cell veto (``CompositeObjectCellVetoEventHandler``, ``event_handler/composite_object_cell_veto_event_handler.py:110-162``
with ``event_handler/abstracts/cell_veto_event_handler.py:162-238``); output files go to a scratch directory.
Recorded:

* the bound tables of the handler (upper and lower derivative bound for every relative cell and direction, as the
  estimator filled them) and the estimator's dipole charge;
* cell-bounding ``send_event_time``: the relative cell, the active unit's charge and velocity, the target units'
  charges, the potential change (``random.expovariate``), the time displacement and the bounding event rate;
* cell-veto ``send_event_time``: the charge factor, the direction and speed, the Walker table's total rate, the
  sampled relative cell, the potential change, the time displacement and the bounding event rate;
* ``send_out_state`` with a target: the units of both composite objects at the event (time-sliced), sorted by
  identifier as the handler sorts them, the active unit's index, whether the local composite object comes first,
  the bounding event rate the thinning draws against, every ``random.uniform`` call (arguments and value) and the
  outcome (rejected, or the unit that became active).
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
    "dipoles_cell_bounding": ("2018_JCP_149_064113/dipoles/cell_bounded.ini", 21, "cell_bounding"),
    "dipoles_cell_veto": ("2018_JCP_149_064113/dipoles/cell_veto.ini", 22, "cell_veto"),
    "water_cell_veto": ("2018_JCP_149_064113/water/coulomb_cell_veto_lj_inverted.ini", 23, "cell_veto"),
}
ACCEPTED = 30   # recorded accepted out-states per configuration
REJECTED = 20   # recorded rejected (thinned) out-states per configuration
TIMES = 60      # recorded event-time calls per configuration
MAX_EVENTS = 400000  # give up on a run after this many calls of the handler


class Stop(Exception):
    pass


def run_one(tree, name, out):
    path, seed, kind = CONFIGS[name]
    os.chdir(os.path.join(tree, "jellyfysh"))
    sys.path.insert(0, tree)
    import logging
    logging.disable(logging.ERROR)
    from jellyfysh.base import factory
    from jellyfysh.base.strings import to_camel_case
    if kind == "cell_bounding":
        from jellyfysh.event_handler import two_composite_object_cell_bounding_potential_event_handler as module
        handler_class = module.TwoCompositeObjectCellBoundingPotentialEventHandler
    else:
        from jellyfysh.event_handler import composite_object_cell_veto_event_handler as module
        handler_class = module.CompositeObjectCellVetoEventHandler

    config = configparser.ConfigParser()
    config.read(os.path.join("config_files", path))
    scratch = tempfile.mkdtemp()
    for section in config.sections():
        if config.has_option(section, "filename") and section != "FactorTypeMaps":
            config.set(section, "filename", os.path.join(scratch, section + ".dat"))
    setting_section = config["HypercubicSetting"]
    record = {"config": path, "kind": kind, "system_length": float(setting_section["system_length"]),
              "beta": float(setting_section["beta"]), "times": [], "out_states": []}

    ctx = {"calls": None, "count": 0}
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

    original_choice = random.choice

    def choice(seq):
        value = original_choice(seq)
        if ctx["calls"] is not None:
            ctx["calls"].append(("choice", [len(seq)], [i for i, entry in enumerate(seq) if entry is value][0]))
        return value
    random.expovariate, random.uniform, random.choice = expovariate, uniform, choice

    def cell_index(cell):
        """The flat index of a cuboid cell: its identifier (x, y, z) with x running fastest."""
        identifier, index, stride = cell.identifier, 0, 1
        for axis, count in enumerate(ctx["cells_per_side"]):
            index += identifier[axis] * stride
            stride *= count
        return index

    def tables(self):
        """upper[cell][direction], lower[cell][direction] over every cell index (None for nearby cells); for the
        cell veto also the Walker tables by bound and direction."""
        if kind == "cell_bounding":
            bounds = self._bounding_potential._derivative_bounds
            estimator = self._bounding_potential._estimator
            upper = {cell_index(cell): list(values) for cell, values in bounds[0].items()}
            lower = {cell_index(cell): list(values) for cell, values in bounds[1].items()}
        else:
            estimator = self._estimator
            upper = {cell_index(cell): [values[d][0] for d in range(3)]
                     for cell, values in self._derivative_bounds.items()}
            lower = {cell_index(cell): [values[d][1] for d in range(3)]
                     for cell, values in self._derivative_bounds.items()}
        cells = self._cells
        total = 1
        for count in cells._cells_per_side:
            total *= count
        result = {"cells_per_side": list(cells._cells_per_side), "cells": total,
                  "upper": [upper.get(c) for c in range(total)], "lower": [lower.get(c) for c in range(total)],
                  "dipole_charge": estimator._dipole_charge}
        if kind == "cell_veto":
            result["walker_upper"] = [walker.total_rate for walker in self._upper_bound_walker]
            result["walker_lower"] = [walker.total_rate for walker in self._lower_bound_walker]
            result["walkers"] = {
                "upper": [walker_record(self, w, d, 0) for d, w in enumerate(self._upper_bound_walker)],
                "lower": [walker_record(self, w, d, 1) for d, w in enumerate(self._lower_bound_walker)]}
        return result

    def walker_record(self, walker, direction, which):
        """The items the handler gave the Walker table (relative cell and rate, in its order: the non-nearby cells
        in cell order with max(bound, 0.0), cell_veto_event_handler.py:148-160) and the table it built (first
        item, first rate, second item or -1)."""
        items, rates = [], []
        for cell in self._cells.yield_cells():
            if cell in self._cells.nearby_cells(self._cells.zero_cell):
                continue
            separation = self._cells.relative_cell(cell, self._cells.zero_cell)
            items.append(cell_index(separation))
            rates.append(max(self._derivative_bounds[separation][direction][which], 0.0))
        table = [[cell_index(entry[0].item), entry[0].rate, cell_index(entry[1].item) if len(entry) > 1 else -1]
                 for entry in walker._table]
        return {"items": items, "rates": rates, "table": table, "mean_rate": walker._mean_rate,
                "total_rate": walker.total_rate}

    def first_call(self):
        if "coulomb" in record:
            return
        ctx["cells_per_side"] = list(self._cells._cells_per_side)
        potential = self._potential
        record["potential"] = type(potential).__name__
        record["lifting_class"] = type(self._lifting).__name__
        record["charge"] = self._charge
        record["coulomb"] = {"alpha": potential._alpha, "fourier_cutoff": potential._fourier_cutoff,
                             "position_cutoff": potential._position_cutoff, "prefactor": potential._prefactor}
        record["tables"] = tables(self)

    def unit_record(unit):
        return {"position": list(unit.position), "charge": unit.charge[record["charge"]]}

    def finish_out(self, entry, calls, state_before):
        local = self._local_leaf_units
        target = self._target_leaf_units
        entry.update(local=[unit_record(u) for u in local], target=[unit_record(u) for u in target],
                     local_first=local[0].identifier[0] < target[0].identifier[0])
        entry["uniform_calls"] = [[args, value] for k, args, value in calls if k == "uniform"]
        units = list(local) + list(target)
        active = [i for i, u in enumerate(local) if u is self._active_leaf_unit]
        entry["active_index"] = active[0]
        moved = [i for i, u in enumerate(units) if u.velocity is not None]
        assert len(moved) == 1
        entry["accepted"] = len(entry["uniform_calls"]) > 1
        entry["new_active"] = moved[0] if entry["accepted"] else -1
        kept = sum(1 for e in record["out_states"] if e["accepted"] == entry["accepted"])
        if kept < (ACCEPTED if entry["accepted"] else REJECTED):
            record["out_states"].append(entry)

    def check_done():
        ctx["count"] += 1
        if (len(record["out_states"]) >= ACCEPTED + REJECTED and len(record["times"]) >= TIMES) or \
                ctx["count"] > MAX_EVENTS:
            raise Stop()

    original_time = handler_class.send_event_time
    original_out = handler_class.send_out_state
    original_slice = handler_class._time_slice_all_units_in_state

    def time_slice(self):
        # called at the end of send_event_time: the active unit's time stamp is still the one before the event
        stamp = self._active_leaf_unit.time_stamp
        ctx["stamp"] = [stamp.quotient, stamp.remainder]
        return original_slice(self)
    handler_class._time_slice_all_units_in_state = time_slice

    from jellyfysh.event_handler import walker as walker_module
    original_sample = walker_module.Walker.sample_cell

    def sample_cell(self):
        value = original_sample(self)
        ctx["relative_cell"] = value
        return value
    walker_module.Walker.sample_cell = sample_cell

    if kind == "cell_bounding":
        def send_event_time(self, in_state):
            ctx["calls"] = []
            try:
                result = original_time(self, in_state)
            finally:
                calls, ctx["calls"] = ctx["calls"], None
            first_call(self)
            velocity = list(self._active_leaf_unit.velocity)
            d = [i for i, v in enumerate(velocity) if v != 0.0][0]
            if len(record["times"]) < TIMES:
                record["times"].append({
                    "relative_cell": cell_index(self._relative_cell), "direction": d, "speed": velocity[d],
                    "active_charge": self._active_leaf_unit.charge[record["charge"]],
                    "target_charges": [u.charge[record["charge"]] for u in self._target_leaf_units],
                    "potential_change": [v for k, _, v in calls if k == "expovariate"][0],
                    "time_stamp": ctx["stamp"], "event_time": [result.quotient, result.remainder],
                    "bounding_event_rate": self._bounding_potential._bounding_event_rate})
            return result

        def send_out_state(self):
            first_call(self)
            entry = {"velocity": list(self._active_leaf_unit.velocity)}
            original_derivative = self._bounding_potential.derivative
            rates = []

            def derivative(*args):
                value = original_derivative(*args)
                rates.append(value)
                return value
            self._bounding_potential.derivative = derivative
            ctx["calls"] = []
            try:
                result = original_out(self)
            finally:
                calls, ctx["calls"] = ctx["calls"], None
                self._bounding_potential.derivative = original_derivative
            if result is not None and rates:
                entry["bounding_event_rate"] = rates[0]
                finish_out(self, entry, calls, None)
            check_done()
            return result
    else:
        def send_event_time(self, in_state):
            ctx["calls"] = []
            try:
                result = original_time(self, in_state)
            finally:
                calls, ctx["calls"] = ctx["calls"], None
            first_call(self)
            event_time, target_cells = result
            velocity = list(self._active_leaf_unit.velocity)
            d = [i for i, v in enumerate(velocity) if v != 0.0][0]
            charge_factor = self._estimator.charge_correction_factor(
                self._active_leaf_unit.charge[record["charge"]])
            walker = (self._upper_bound_walker if charge_factor > 0.0 else self._lower_bound_walker)[d]
            if len(record["times"]) < TIMES:
                record["times"].append({
                    "direction": d, "speed": velocity[d], "charge_factor": charge_factor,
                    "walker_total_rate": walker.total_rate,
                    "potential_change": [v for k, _, v in calls if k == "expovariate"][0],
                    "time_stamp": ctx["stamp"], "event_time": [event_time.quotient, event_time.remainder],
                    "relative_cell": cell_index(ctx["relative_cell"]),
                    "walker_choice": [v for k, _, v in calls if k == "choice"][0],
                    "walker_uniform": [v for k, _, v in calls if k == "uniform"][0],
                    "bounding_event_rate": self._bounding_event_rate})
            return result

        def send_out_state(self, target_cnode):
            first_call(self)
            entry = {"velocity": list(self._active_leaf_unit.velocity),
                     "bounding_event_rate": self._bounding_event_rate}
            ctx["calls"] = []
            try:
                result = original_out(self, target_cnode)
            finally:
                calls, ctx["calls"] = ctx["calls"], None
            if target_cnode is not None:
                finish_out(self, entry, calls, None)
            check_done()
            return result

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
    path = os.path.join(HERE, "composite_cell_events.json")
    with open(path, "w") as handle:
        json.dump({"source": "reference runs of its molecular cell-bounding and cell-veto configurations",
                   "systems": records}, handle)
        handle.write("\n")
    print("wrote", path)


if __name__ == "__main__":
    from _tree import tree_argument
    if len(sys.argv) > 1 and sys.argv[1] == "--one":
        run_one(sys.argv[2], sys.argv[3], sys.argv[4])
    else:
        main(tree_argument(sys.argv))
