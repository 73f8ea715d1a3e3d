"""Record estimator samples of long runs of the reference's own event loop as golden fixtures.

Run in a container that holds the JeLLyFysh source tree with its cffi extensions built:

    python tests/golden/make_reference_estimators.py /path/to/jellyfysh/tree [name ...]

The reference runs unchanged with its own random numbers (Python's ``random``, seeded) from the INI
configuration that ``make_reference_trajectories.py`` writes for the same system; only the initial positions are
injected (``AtomRandomNodeCreator.fill_root_node``), and every commit of the state handler is observed:

* at every end-of-chain event (times k * chain_time) the positions of all units are sampled: potential energy
  (Lennard-Jones) and the pair-distance histogram (``jellyfysh_gb300.estimators``);
* at every accepted lifting the separation target - active along the direction of motion is added to the
  excess displacement of the current chain.

Sixteen independent runs (own Python seed, own initial jitter, burn-in of `burn_in` chains) give independent
blocks for the errors.  The fixture holds per-run, per-chain samples (energy, lifting sum) and per-run
histograms, from which the tests compute the estimators and their errors exactly as they do for the GPU engine and
the oracle.
"""
import json
import os
import random
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import make_reference_trajectories as trajectories  # noqa: E402

BINS = 40
RUNS = 16  # independent runs of the reference (own Python seed and initial jitter): the blocks of the errors
SYSTEMS = {
    "lennard_jones_n64_cell_veto": dict(trajectories.SYSTEMS["lennard_jones_n64_cell_veto"], burn_in=200,
                                        samples=240, r_max_fraction=0.5, python_seed=2024),
    "hard_spheres_n64": dict(trajectories.SYSTEMS["hard_spheres_n64"], burn_in=400, samples=1000,
                             r_max_fraction=0.5, python_seed=2025),
}


def run_one(tree: str, name: str, run: int, out: str) -> None:
    spec = dict(SYSTEMS[name], seed=SYSTEMS[name]["seed"] + 1000 * run)
    sys.path.insert(0, tree)
    import configparser
    import logging
    logging.disable(logging.ERROR)
    from jellyfysh_gb300 import estimators
    length, positions, charges = trajectories.initial_state(spec)
    from jellyfysh.base import factory
    from jellyfysh.base.exceptions import EndOfRun
    from jellyfysh.base.particle import Particle
    from jellyfysh.base.strings import to_camel_case
    from jellyfysh.input_output_handler.input_handler.random_node_creator import atom_random_node_creator
    from jellyfysh.state_handler.tree_state_handler import TreeStateHandler
    from jellyfysh.scheduler.heap_scheduler.heap_scheduler import HeapScheduler

    random.seed(spec["python_seed"] + run)
    n = spec["n"]
    r_max = spec["r_max_fraction"] * length
    queue = list(range(n))

    def fill_root_node(self, node):
        i = queue.pop(0)
        node.value = Particle([float(v) for v in positions[i]], {})
    atom_random_node_creator.AtomRandomNodeCreator.fill_root_node = fill_root_node

    ctx = {"winner": None, "depth": 0, "active": None, "chains": 0, "lift": 0.0, "liftings": 0}
    original_succeeding = HeapScheduler.get_succeeding_event

    def get_succeeding_event(self):
        handler = original_succeeding(self)
        ctx["winner"] = handler
        return handler
    HeapScheduler.get_succeeding_event = get_succeeding_event

    samples = {"energy": [], "lift": [], "liftings": []}
    histogram = np.zeros(BINS, dtype=np.int64)

    class Stop(Exception):
        pass

    original_insert = TreeStateHandler.insert_into_global_state

    def insert_into_global_state(self, out_state):
        ctx["depth"] += 1
        try:
            result = original_insert(self, out_state)
        finally:
            ctx["depth"] -= 1
        if ctx["depth"] > 0:
            return result
        active = self.extract_active_global_state()[0].value
        active_id = active.identifier[0]
        direction = [i for i, v in enumerate(active.velocity) if v != 0.0][0]
        winner_name = type(ctx["winner"]).__name__
        moved = ctx["active"]
        if winner_name == "SingleIndependentActivePeriodicDirectionEndOfChainEventHandler":
            ctx["chains"] += 1
            if ctx["chains"] > spec["burn_in"]:
                config = np.array([self.extract_from_global_state((i,)).value.position for i in range(n)],
                                  dtype=np.float64)
                samples["energy"].append(estimators.lennard_jones_energy(config, length)
                                         if spec["potential"] == "lennard_jones" else 0.0)
                samples["lift"].append(ctx["lift"])
                samples["liftings"].append(ctx["liftings"])
                histogram[:] += estimators.pair_histogram(config, length, BINS, r_max)
                if ctx["chains"] - spec["burn_in"] >= spec["samples"]:
                    raise Stop()
            ctx["lift"] = 0.0
            ctx["liftings"] = 0
        elif moved is not None and active_id != moved:
            # accepted lifting: separation target - active along the direction, as separation_vector computes it
            target = self.extract_from_global_state((active_id,)).value.position[direction]
            source = self.extract_from_global_state((moved,)).value.position[direction]
            ctx["lift"] += ((target - source) + length / 2.0) % length - length / 2.0
            ctx["liftings"] += 1
        ctx["active"] = active_id
        return result
    TreeStateHandler.insert_into_global_state = insert_into_global_state

    config = configparser.ConfigParser()
    config.read_string(trajectories.config_text(spec, length))
    factory.build_from_config(config, to_camel_case(config.get("Run", "setting")), "jellyfysh.setting")
    mediator = factory.build_from_config(config, to_camel_case(config.get("Run", "mediator")), "jellyfysh.mediator")
    start = time.time()
    try:
        mediator.run()
    except (Stop, EndOfRun):
        pass
    np.savez(out, energy=np.array(samples["energy"]), lift=np.array(samples["lift"]),
             liftings=np.array(samples["liftings"]), histogram=histogram, length=length, r_max=r_max)
    print("%s run %d: %d chain samples in %.0f s" % (name, run, len(samples["energy"]), time.time() - start))


def main(tree: str, names) -> None:
    import concurrent.futures
    import tempfile
    with tempfile.TemporaryDirectory() as scratch:
        def one(job):
            name, run = job
            out = os.path.join(scratch, "%s_%d.npz" % (name, run))
            subprocess.run([sys.executable, os.path.abspath(__file__), "--one", tree, name, str(run), out],
                           check=True)
            return out
        jobs = [(name, run) for name in names for run in range(RUNS)]
        with concurrent.futures.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as pool:
            outs = dict(zip(jobs, pool.map(one, jobs)))
        for name in names:
            runs = [np.load(outs[(name, run)]) for run in range(RUNS)]
            spec = dict(SYSTEMS[name], system_length=float(runs[0]["length"]), r_max=float(runs[0]["r_max"]),
                        bins=BINS, runs=RUNS, speed=1.0)
            path = os.path.join(HERE, "estimators_%s.npz" % name)
            np.savez_compressed(path, energy=np.array([r["energy"] for r in runs]),
                                lift=np.array([r["lift"] for r in runs]),
                                liftings=np.array([r["liftings"] for r in runs]),
                                histograms=np.array([r["histogram"] for r in runs]), spec=json.dumps(spec))
            print("%s: %d runs -> %s" % (name, RUNS, path))


if __name__ == "__main__":
    from _tree import tree_argument
    if len(sys.argv) > 1 and sys.argv[1] == "--one":
        run_one(sys.argv[2], sys.argv[3], int(sys.argv[4]), sys.argv[5])
    else:
        tree_path = tree_argument(sys.argv)
        main(tree_path, sys.argv[2:] or list(SYSTEMS))
