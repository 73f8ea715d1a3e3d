"""Record event-by-event trajectories of the reference's own event loop as golden fixtures.

Run in a container that holds the JeLLyFysh source tree with its cffi extensions built:

    python tests/golden/make_reference_trajectories.py /path/to/jellyfysh/tree [name ...]

For every system below the script writes the reference's INI configuration (in the reference's own vocabulary),
builds the mediator with the reference's factory (``jellyfysh/run.py:181-183``) and runs
``SingleProcessMediator.run`` (``jellyfysh/mediator/single_process_mediator.py:91-156``) unchanged.  Three things are
replaced around it:

* the initial state: ``AtomRandomNodeCreator.fill_root_node`` places the seeded synthetic positions and charges of
  ``jellyfysh_gb300.systems`` instead of random ones;
* the random numbers: every ``random`` call site on the path returns the keyed draw of the oracle's generator
  (``oracle.draw``) for (event index, kind, target), so the GPU engine and the oracle see the same numbers;
* the output: every commit of the state handler is logged (winner, target, lifting outcome, event time, committed
  position of the moved unit) until the requested number of events.

Each system runs in its own interpreter because the reference keeps its setting in module globals.
"""
import json
import math
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

SYSTEMS = {
    "hard_spheres_n64": dict(potential="hard_sphere", n=64, radius=0.1, system_length=1.0, cells_per_side=5,
                             neighbor_layers=1, chain_time=0.3, beta=1.0, far="none", seed=11, events=3000,
                             state="rsa"),
    "lennard_jones_n64_cell_veto": dict(potential="lennard_jones", n=64, density=0.8, cells_per_side=4,
                                        neighbor_layers=1, chain_time=2.0, beta=1.0 / 1.2, far="cell_veto", seed=12,
                                        events=2500, state="sc", estimator_prefactor=1.5, estimator_points=10),
    "lennard_jones_n64_cell_bounding": dict(potential="lennard_jones", n=64, density=0.8, cells_per_side=4,
                                            neighbor_layers=1, chain_time=2.0, beta=1.0 / 1.2,
                                            far="cell_bounding", seed=13, events=1500, state="sc",
                                            estimator_prefactor=1.5, estimator_points=10),
    "lennard_jones_n128_two_layers_cell_veto": dict(potential="lennard_jones", n=128, density=0.8, cells_per_side=6,
                                                    neighbor_layers=2, chain_time=2.0, beta=1.0 / 1.2,
                                                    far="cell_veto", seed=15, events=1500, state="sc",
                                                    estimator_prefactor=1.5, estimator_points=10),
    # the geometry of the batched Lennard-Jones workload (N = 1024, density 0.8, 12^3 cells, three neighbour layers)
    "lennard_jones_n1024_three_layers_cell_veto": dict(potential="lennard_jones", n=1024, density=0.8,
                                                       cells_per_side=12, neighbor_layers=3, chain_time=2.0,
                                                       beta=1.0 / 1.2, far="cell_veto", seed=16, events=1000,
                                                       state="sc", estimator_prefactor=1.5, estimator_points=10),
    # three neighbour layers with the cell-bounding far field at N = 512 (9^3 cells): the reference deep-copies one
    # event handler per cell, and at N = 1024 (12^3 cells) its copies outgrow the memory of the recording machine
    "lennard_jones_n512_three_layers_cell_bounding": dict(potential="lennard_jones", n=512, density=0.8,
                                                          cells_per_side=9, neighbor_layers=3, chain_time=2.0,
                                                          beta=1.0 / 1.2, far="cell_bounding", seed=17,
                                                          events=400, state="sc", estimator_prefactor=1.5,
                                                          estimator_points=10),
    "coulomb_n8_cell_veto": dict(potential="coulomb", n=8, radius=0.05, system_length=1.0, cells_per_side=4,
                                 neighbor_layers=1, chain_time=0.7, beta=1.0, far="cell_veto", seed=14, events=2500,
                                 state="rsa_charged", estimator_prefactor=1.0, estimator_points=10),
}

PAIR_SECTIONS = """
[{Name}Nearby]
create = {create}
trash = {create}
internal_state_label = single_active_cell_occupancy
event_handler = {handler}
number_event_handlers = {nearby_handlers}

[{Name}Surplus]
create = {create}
trash = {create}
internal_state_label = single_active_cell_occupancy
event_handler = {handler}
number_event_handlers = {surplus_handlers}
"""


def config_text(spec: dict, system_length: float) -> str:
    far = spec["far"]
    pair_tags = []
    sections = []
    taggers = []
    if spec["potential"] in ("hard_sphere", "lennard_jones"):
        handler = "two_leaf_unit_event_handler"
        pair_tags = ["pair_nearby", "pair_surplus"]
        taggers += ["pair_nearby (excluded_cells_tagger)", "pair_surplus (surplus_cells_tagger)"]
    else:
        pair_tags = ["hardcore_nearby", "hardcore_surplus", "coulomb_nearby", "coulomb_surplus"]
        taggers += ["hardcore_nearby (excluded_cells_tagger)", "hardcore_surplus (surplus_cells_tagger)",
                    "coulomb_nearby (excluded_cells_tagger)", "coulomb_surplus (surplus_cells_tagger)"]
    far_tag = []
    if far == "cell_veto":
        far_tag = ["far_cell_veto"]
        taggers.append("far_cell_veto (cell_veto_tagger)")
    elif far == "cell_bounding":
        far_tag = ["far_cell_bounding"]
        taggers.append("far_cell_bounding (cell_bounding_potential_tagger)")
    taggers += ["cell_boundary (cell_boundary_tagger)", "end_of_chain (active_global_state_in_state_tagger)",
                "end_of_run (no_in_state_tagger)", "start_of_run (no_in_state_tagger)"]
    create = ", ".join(pair_tags + far_tag + ["cell_boundary"])
    ncells = spec["cells_per_side"] ** 3
    n = spec["n"]
    text = """
[Run]
mediator = single_process_mediator
setting = hypercubic_setting

[HypercubicSetting]
system_length = {L!r}
beta = {beta!r}
dimension = 3

[SingleProcessMediator]
state_handler = tree_state_handler
scheduler = heap_scheduler
activator = tag_activator
input_output_handler = input_output_handler

[TagActivator]
taggers = {taggers}
internal_states = single_active_cell_occupancy

[SingleActiveCellOccupancy]
cells = cuboid_periodic_cells
cell_level = 1
maximum_number_occupants = 1

[CuboidPeriodicCells]
cells_per_side = {m}
neighbor_layers = {layers}

[CellBoundary]
create = {create}
trash = {create}
internal_state_label = single_active_cell_occupancy
event_handler = cell_boundary_event_handler

[EndOfChain]
create = end_of_chain, {create}
trash = end_of_chain, {create}
event_handler = single_independent_active_periodic_direction_end_of_chain_event_handler

[SingleIndependentActivePeriodicDirectionEndOfChainEventHandler]
chain_time = {chain_time!r}

[EndOfRun]
create = end_of_run
trash = end_of_chain, {create}, end_of_run
event_handler = final_time_end_of_run_event_handler

[FinalTimeEndOfRunEventHandler]
end_of_run_time = 1000000000.0

[StartOfRun]
trash = start_of_run
create = end_of_chain, {create}, end_of_run
event_handler = initial_chain_start_of_run_event_handler

[InitialChainStartOfRunEventHandler]
initial_direction_of_motion = 0
speed = 1.0
initial_active_identifier = 0

[TreeStateHandler]
physical_state = tree_physical_state
lifting_state = tree_lifting_state

[InputOutputHandler]
input_handler = random_input_handler

[RandomInputHandler]
random_node_creator = atom_random_node_creator
number_of_root_nodes = {n}
""".format(L=system_length, beta=spec["beta"], taggers=",\n    ".join(taggers), m=spec["cells_per_side"],
           layers=spec["neighbor_layers"], create=create, chain_time=spec["chain_time"], n=n)
    if spec["potential"] == "hard_sphere":
        text += PAIR_SECTIONS.format(Name="Pair", create=create, handler="two_leaf_unit_event_handler",
                                     nearby_handlers=ncells, surplus_handlers=n)
        text += "\n[TwoLeafUnitEventHandler]\npotential = hard_sphere_potential\n"
        text += "\n[HardSpherePotential]\nradius = %r\n" % spec["radius"]
    elif spec["potential"] == "lennard_jones":
        text += PAIR_SECTIONS.format(Name="Pair", create=create, handler="two_leaf_unit_event_handler",
                                     nearby_handlers=ncells, surplus_handlers=n)
        text += "\n[TwoLeafUnitEventHandler]\npotential = lennard_jones_potential\n"
        text += "\n[LennardJonesPotential]\nprefactor = 1.0\ncharacteristic_length = 1.0\n"
        text += ("\n[InnerPointEstimator]\npotential = lennard_jones_potential\nprefactor = %r\npoints_per_side = %d\n"
                 % (spec["estimator_prefactor"], spec["estimator_points"]))
    else:
        text += PAIR_SECTIONS.format(Name="Hardcore", create=create, handler="two_leaf_unit_event_handler",
                                     nearby_handlers=ncells, surplus_handlers=n)
        text += PAIR_SECTIONS.format(Name="Coulomb", create=create,
                                     handler="two_leaf_unit_bounding_potential_event_handler",
                                     nearby_handlers=ncells, surplus_handlers=n)
        text += "\n[TwoLeafUnitEventHandler]\npotential = hard_sphere_potential\n"
        text += "\n[HardSpherePotential]\nradius = %r\n" % spec["radius"]
        text += ("\n[TwoLeafUnitBoundingPotentialEventHandler]\npotential = merged_image_coulomb_potential\n"
                 "bounding_potential = inverse_power_coulomb_bounding_potential\ncharge = electric_charge\n")
        text += "\n[MergedImageCoulombPotential]\nalpha = 3.45\nfourier_cutoff = 6\nposition_cutoff = 2\nprefactor = 1.0\n"
        text += "\n[InversePowerCoulombBoundingPotential]\nprefactor = 1.5837\n"
        text += ("\n[InnerPointEstimator]\npotential = merged_image_coulomb_potential\nprefactor = %r\n"
                 "points_per_side = %d\ntarget_charge = 1.0\n" % (spec["estimator_prefactor"], spec["estimator_points"]))
    if far == "cell_veto":
        text += """
[FarCellVeto]
create = {create}
trash = {create}
event_handler = leaf_unit_cell_veto_event_handler
internal_state_label = single_active_cell_occupancy

[LeafUnitCellVetoEventHandler]
estimator = inner_point_estimator
""".format(create=create)
        if spec["potential"] == "coulomb":
            text += "charge = electric_charge\n"
    elif far == "cell_bounding":
        text += """
[FarCellBounding]
create = {create}
trash = {create}
event_handler = two_leaf_unit_cell_bounding_potential_event_handler
number_event_handlers = {ncells}
internal_state_label = single_active_cell_occupancy

[TwoLeafUnitCellBoundingPotentialEventHandler]
potential = lennard_jones_potential
bounding_potential = cell_bounding_potential

[CellBoundingPotential]
estimator = inner_point_estimator
""".format(create=create, ncells=ncells)
    return text


def initial_state(spec: dict):
    sys.path.insert(0, ROOT)
    from jellyfysh_gb300 import systems
    rng = np.random.default_rng(spec["seed"])
    charges = None
    if spec["state"] == "rsa":
        length = spec["system_length"]
        positions = systems.random_sequential_addition(spec["n"], spec["radius"], length, rng)
    elif spec["state"] == "rsa_charged":
        length = spec["system_length"]
        positions = systems.random_sequential_addition(spec["n"], spec["radius"], length, rng)
        charges = systems.alternating_charges(spec["n"])
    else:
        length = systems.lennard_jones_box(spec["n"], spec["density"])
        positions = systems.simple_cubic_jitter(spec["n"], length, 0.05, rng)
    return length, positions, charges


def run_one(tree: str, name: str) -> None:
    spec = SYSTEMS[name]
    structured, positions, final, charges, length, key = record(tree, spec)
    out = os.path.join(HERE, "trajectory_%s.npz" % name)
    np.savez_compressed(out, events=structured, initial=positions, final=final,
                        charges=np.zeros(0) if charges is None else charges,
                        spec=json.dumps(dict(spec, system_length=length, rng_key=key)))
    print("%s: %d events, kinds %s -> %s" % (name, len(structured), np.bincount(structured["kind"], minlength=8), out))


def record(tree: str, spec: dict, transform=None, prepare=None):
    """Run the reference's mediator on the system `spec` with the keyed random numbers and log every commit.
    `transform` (optional) rewrites the configuration text; `prepare(context)` (optional) is called before the run
    with the event-index function, the chain's key and beta, so that other event handlers draw the same numbers.
    Returns (events, initial positions, final positions, charges, box length, key)."""
    sys.path.insert(0, tree)
    sys.path.insert(0, ROOT)
    import configparser
    import logging
    logging.disable(logging.ERROR)
    import oracle
    length, positions, charges = initial_state(spec)
    key = oracle.chain_key(spec["seed"], 0)
    from jellyfysh.base import factory
    from jellyfysh.base.exceptions import EndOfRun
    from jellyfysh.base.particle import Particle
    from jellyfysh.base.strings import to_camel_case
    from jellyfysh.input_output_handler.input_handler.random_node_creator import atom_random_node_creator
    from jellyfysh.state_handler.tree_state_handler import TreeStateHandler
    from jellyfysh.scheduler.heap_scheduler.heap_scheduler import HeapScheduler
    import jellyfysh.event_handler.two_leaf_unit_event_handler as m_pair
    import jellyfysh.event_handler.two_leaf_unit_bounding_potential_event_handler as m_bounded
    import jellyfysh.event_handler.two_leaf_unit_cell_bounding_potential_event_handler as m_cell_bounding
    import jellyfysh.event_handler.abstracts.event_handler_with_bounding_potential as m_thin
    import jellyfysh.event_handler.abstracts.cell_veto_event_handler as m_veto
    import jellyfysh.event_handler.walker as m_walker
    import jellyfysh.event_handler.single_independent_active_periodic_direction_end_of_chain_event_handler as m_eoc

    ctx = {"commits": 0, "target": None, "winner": None}
    beta = spec["beta"]

    def event_index():
        return ctx["commits"] - 1

    class PairRandom:
        @staticmethod
        def expovariate(lambd):
            assert lambd == beta
            return oracle.expovariate(oracle.draw(key, event_index(), oracle.RNG_PAIR, ctx["target"]), lambd)

    class ThinRandom:
        @staticmethod
        def uniform(a, b):
            u = oracle.uniform(oracle.draw(key, event_index(), oracle.RNG_THIN, 0))
            return a + (b - a) * u

    class VetoRandom:
        @staticmethod
        def expovariate(lambd):
            assert lambd == beta
            return oracle.expovariate(oracle.draw(key, event_index(), oracle.RNG_VETO_TIME, 0), lambd)

    class WalkerRandom:
        @staticmethod
        def choice(sequence):
            return sequence[oracle.randbelow(oracle.draw(key, event_index(), oracle.RNG_VETO_CHOICE, 0),
                                             len(sequence))]

        @staticmethod
        def uniform(a, b):
            u = oracle.uniform(oracle.draw(key, event_index(), oracle.RNG_VETO_UNIFORM, 0))
            return a + (b - a) * u

    def eoc_randint(a, b):
        assert a == 0
        return oracle.randbelow(oracle.draw(key, event_index(), oracle.RNG_NEW_ACTIVE, 0), b + 1)

    m_pair.random = PairRandom
    m_bounded.random = PairRandom
    m_cell_bounding.random = PairRandom
    m_thin.random = ThinRandom
    m_veto.random = VetoRandom
    m_walker.random = WalkerRandom
    m_eoc.randint = eoc_randint

    def with_target(cls):
        original = cls.send_event_time

        def send_event_time(self, in_state):
            ctx["target"] = in_state[1].value.identifier[0]
            return original(self, in_state)
        cls.send_event_time = send_event_time

    with_target(m_pair.TwoLeafUnitEventHandler)
    with_target(m_bounded.TwoLeafUnitBoundingPotentialEventHandler)
    with_target(m_cell_bounding.TwoLeafUnitCellBoundingPotentialEventHandler)

    queue = list(range(spec["n"]))

    def fill_root_node(self, node):
        i = queue.pop(0)
        charge = {} if charges is None else {"electric_charge": float(charges[i])}
        node.value = Particle([float(v) for v in positions[i]], charge)
    atom_random_node_creator.AtomRandomNodeCreator.fill_root_node = fill_root_node

    original_succeeding = HeapScheduler.get_succeeding_event

    def get_succeeding_event(self):
        handler = original_succeeding(self)
        ctx["winner"] = handler
        return handler
    HeapScheduler.get_succeeding_event = get_succeeding_event

    log = []
    state = {"handler": None, "active": None, "direction": None}
    kinds = {"TwoLeafUnitEventHandler": oracle.EV_HARDCORE if spec["potential"] == "coulomb" else oracle.EV_PAIR,
             "TwoLeafUnitBoundingPotentialEventHandler": oracle.EV_BOUNDED,
             "TwoLeafUnitCellBoundingPotentialEventHandler": oracle.EV_CELL_BOUNDING,
             "LeafUnitCellVetoEventHandler": oracle.EV_CELL_VETO,
             "CellBoundaryEventHandler": oracle.EV_BOUNDARY,
             "SingleIndependentActivePeriodicDirectionEndOfChainEventHandler": oracle.EV_END_OF_CHAIN}

    class Stop(Exception):
        pass

    original_insert = TreeStateHandler.insert_into_global_state

    def insert_into_global_state(self, out_state):
        ctx["depth"] = ctx.get("depth", 0) + 1
        try:
            result = original_insert(self, out_state)
        finally:
            ctx["depth"] -= 1
        if ctx["depth"] > 0:
            return result
        ctx["commits"] += 1
        active = self.extract_active_global_state()[0].value
        active_id = active.identifier[0]
        direction = [i for i, v in enumerate(active.velocity) if v != 0.0][0]
        winner = ctx["winner"]
        name_of = type(winner).__name__
        if name_of in kinds:
            moved = state["active"]
            kind = kinds[name_of]
            target = -1
            accepted = 0
            if hasattr(winner, "_target_index"):  # an event handler of a whole neighbourhood
                target = winner._leaf_units[winner._target_index].identifier[0]
                accepted = int(active_id != moved)
            elif kind in (oracle.EV_PAIR, oracle.EV_HARDCORE, oracle.EV_BOUNDED, oracle.EV_CELL_BOUNDING):
                target = winner._leaf_units[winner._active_leaf_unit_index ^ 1].identifier[0]
                accepted = int(active_id != moved)
            elif kind == oracle.EV_CELL_VETO:
                if len(winner._leaf_units) == 2:
                    target = winner._leaf_units[winner._active_leaf_unit_index ^ 1].identifier[0]
                accepted = int(active_id != moved)
            elif kind == oracle.EV_END_OF_CHAIN:
                target = active_id
                accepted = 1
            moved_unit = self.extract_from_global_state((moved,)).value
            time = winner._event_time
            log.append((kind, moved, target, active_id, direction, accepted, time.quotient, time.remainder,
                        moved_unit.position[0], moved_unit.position[1], moved_unit.position[2]))
            if len(log) >= spec["events"]:
                raise Stop()
        state["active"] = active_id
        state["direction"] = direction
        return result
    TreeStateHandler.insert_into_global_state = insert_into_global_state

    if prepare is not None:
        prepare({"event_index": event_index, "key": key, "beta": beta, "kinds": kinds})
    text = config_text(spec, length)
    config = configparser.ConfigParser()
    config.read_string(transform(text) if transform is not None else text)
    factory.build_from_config(config, to_camel_case(config.get("Run", "setting")), "jellyfysh.setting")
    mediator = factory.build_from_config(config, to_camel_case(config.get("Run", "mediator")), "jellyfysh.mediator")
    try:
        mediator.run()
    except Stop:
        pass
    except EndOfRun:
        pass
    final = np.array([mediator._state_handler.extract_from_global_state((i,)).value.position
                      for i in range(spec["n"])], dtype=np.float64)
    structured = np.zeros(len(log), dtype=oracle.EVENT_DTYPE)
    for field_index, field in enumerate(oracle.EVENT_DTYPE.names):
        structured[field] = [row[field_index] for row in log]
    return structured, positions, final, charges, length, key


def main(tree: str, names) -> None:
    for name in names:
        subprocess.run([sys.executable, os.path.abspath(__file__), "--one", tree, name], check=True)


if __name__ == "__main__":
    from _tree import tree_argument
    if len(sys.argv) > 1 and sys.argv[1] == "--one":
        run_one(sys.argv[2], sys.argv[3])
    else:
        tree_path = tree_argument(sys.argv)
        main(tree_path, sys.argv[2:] or list(SYSTEMS))
