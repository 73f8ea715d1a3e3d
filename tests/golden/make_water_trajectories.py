"""Record event-by-event trajectories of the reference's event loop for flexible water as golden fixtures.

Run in a container that holds the JeLLyFysh source tree with its cffi extensions built:

    python tests/golden/make_water_trajectories.py /path/to/jellyfysh/tree [name ...]

The system is written in the reference's own vocabulary: water molecules as composite objects of three point charges
(hydrogen, oxygen, hydrogen), a factor-set file (``activator/tagger/factor_type_maps.py``) with harmonic O–H and
H–H bonds (``DisplacedEvenPowerPotential``), Lennard-Jones between oxygens and one Coulomb factor per pair of
molecules (``TwoCompositeObjectSummedBoundingPotentialEventHandler``: merged-image Coulomb bounded by the
inverse-power Coulomb bound, inside-first lifting), all taken by ``FactorTypeMapInStateTagger`` for every pair of
molecules, and the periodic-direction end of chain.  ``SingleProcessMediator.run`` runs unchanged; three things
are replaced around it, as for the atomic trajectories:

* the initial state: ``WaterRandomNodeCreator.fill_root_node`` places the molecules of
  ``jellyfysh_gb300.systems.water_lattice``;
* the random numbers: every ``random`` call site on the path returns the keyed draw of the oracle's generator
  (``oracle.draw``) for (event index, kind, target): the potential change of a bond or Lennard-Jones pair is keyed
  by its target unit (kind PAIR), the three potential changes of a Coulomb factor by the target molecule's units
  (kind COMPOSITE), the thinning draw by kind THIN, the lifting draw by kind LIFT, the end of chain's two integers
  by kind NEW_ACTIVE (0: molecule, 1: unit);
* the output: every committed event is logged (kind, moved unit, target, new active unit, direction, thinning
  outcome, event time, committed position of the moved unit).

One line of the reference's factor enumeration is amended (see ``run_one``): its local factor type map raises
KeyError for an active unit that a local factor type does not name, which the H–H bond needs.

Unit index of atom t of molecule m: 3 m + t.  Each system runs in its own interpreter.
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

KILOCALORIE_PER_MOLE_KELVIN = 0.0019872041
WATER = dict(oh_r0=1.0, oh_prefactor=1059.0 / 2.0, hh_r0=1.633, hh_prefactor=684.0 / 2.0,
             lj_prefactor=4.0 * 0.1554, lj_sigma=3.166, coulomb_prefactor=332.0637,
             bound_prefactor=1.6 * 332.0637, alpha=3.45, fourier_cutoff=6, position_cutoff=2,
             charge_oxygen=-0.82, charge_hydrogen=0.41, beta=1.0 / (KILOCALORIE_PER_MOLE_KELVIN * 300.0),
             chain_time=2.0, speed=1.0, initial_active=1, initial_direction=0, lifting="inside_first")
SYSTEMS = {
    "water_n8": dict(WATER, molecules_per_side=2, system_length=12.42 / 2.0, seed=21, events=2500),
    "water_n64": dict(WATER, molecules_per_side=4, system_length=12.42, seed=22, events=4000),
}

FACTORS = """[0, 1], HarmonicOh
[1, 2], HarmonicOh
[0, 2], HarmonicHh
[1, 4], LennardJones
[0, 1, 2, 3, 4, 5], Coulomb
"""

TAGGERS = ["harmonic_oh", "harmonic_hh", "lennard_jones", "coulomb"]


def config_text(spec, factor_file):
    molecules = spec["molecules_per_side"] ** 3
    tags = ", ".join(TAGGERS)
    handlers = {"harmonic_oh": ("harmonic_oh_event_handler (two_leaf_unit_event_handler)", 2),
                "harmonic_hh": ("harmonic_hh_event_handler (two_leaf_unit_event_handler)", 1),
                "lennard_jones": ("lennard_jones_event_handler (two_leaf_unit_event_handler)", molecules - 1),
                "coulomb": ("two_composite_object_summed_bounding_potential_event_handler", molecules - 1)}
    sections = []
    for tag in TAGGERS:
        handler, count = handlers[tag]
        sections.append("[%s]\ncreate = %s\ntrash = %s\nevent_handler = %s\nnumber_event_handlers = %d\n"
                        "factor_type_maps = factor_type_maps\n" % (
                            "".join(p.capitalize() for p in tag.split("_")), tags, tags, handler, count))
    lifting = spec["lifting"] + "_lifting"
    return """
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
taggers =
    harmonic_oh (factor_type_map_in_state_tagger),
    harmonic_hh (factor_type_map_in_state_tagger),
    lennard_jones (factor_type_map_in_state_tagger),
    coulomb (factor_type_map_in_state_tagger),
    end_of_chain (active_global_state_in_state_tagger),
    end_of_run (no_in_state_tagger),
    start_of_run (no_in_state_tagger)

[FactorTypeMaps]
filename = {factor_file}

{sections}
[HarmonicOhEventHandler]
potential = harmonic_oh_potential (displaced_even_power_potential)

[HarmonicOhPotential]
equilibrium_separation = {oh_r0!r}
prefactor = {oh_prefactor!r}
power = 2

[HarmonicHhEventHandler]
potential = harmonic_hh_potential (displaced_even_power_potential)

[HarmonicHhPotential]
equilibrium_separation = {hh_r0!r}
prefactor = {hh_prefactor!r}
power = 2

[LennardJonesEventHandler]
potential = lennard_jones_potential

[LennardJonesPotential]
prefactor = {lj_prefactor!r}
characteristic_length = {lj_sigma!r}

[TwoCompositeObjectSummedBoundingPotentialEventHandler]
potential = merged_image_coulomb_potential
bounding_potential = inverse_power_coulomb_bounding_potential
lifting = {lifting}
charge = electric_charge

[MergedImageCoulombPotential]
prefactor = {coulomb_prefactor!r}
alpha = {alpha!r}
fourier_cutoff = {fourier_cutoff}
position_cutoff = {position_cutoff}

[InversePowerCoulombBoundingPotential]
prefactor = {bound_prefactor!r}

[EndOfChain]
create = end_of_chain, {tags}
trash = end_of_chain, {tags}
event_handler = single_independent_active_periodic_direction_end_of_chain_event_handler

[SingleIndependentActivePeriodicDirectionEndOfChainEventHandler]
chain_time = {chain_time!r}

[EndOfRun]
create = end_of_run
trash = end_of_chain, {tags}, end_of_run
event_handler = final_time_end_of_run_event_handler

[FinalTimeEndOfRunEventHandler]
end_of_run_time = 1e9

[StartOfRun]
trash = start_of_run
create = end_of_chain, {tags}, end_of_run
event_handler = initial_chain_start_of_run_event_handler

[InitialChainStartOfRunEventHandler]
initial_direction_of_motion = {initial_direction}
speed = {speed!r}
initial_active_identifier = 0, {initial_active}

[TreeStateHandler]
physical_state = tree_physical_state
lifting_state = tree_lifting_state

[InputOutputHandler]
input_handler = random_input_handler

[RandomInputHandler]
random_node_creator = water_random_node_creator
number_of_root_nodes = {molecules}

[WaterRandomNodeCreator]
charge_values = electric_charge_values (charge_values)

[ElectricChargeValues]
charge_name = electric_charge
charge_values = {charge_hydrogen!r}, {charge_oxygen!r}, {charge_hydrogen!r}
""".format(L=float(spec["system_length"]), factor_file=factor_file, sections="\n".join(sections), tags=tags,
           lifting=lifting, molecules=molecules, **{k: v for k, v in spec.items() if k != "lifting"})


def initial_state(spec):
    sys.path.insert(0, ROOT)
    from jellyfysh_gb300 import systems
    rng = np.random.default_rng(spec["seed"])
    return systems.water_lattice(spec["molecules_per_side"], spec["system_length"], spec["oh_r0"], spec["hh_r0"], rng,
                                 spec["charge_oxygen"], spec["charge_hydrogen"])


def run_one(tree, name):
    spec = SYSTEMS[name]
    sys.path.insert(0, tree)
    sys.path.insert(0, ROOT)
    import configparser
    import logging
    logging.disable(logging.ERROR)
    import oracle
    positions, charges = initial_state(spec)
    key = oracle.chain_key(spec["seed"], 0)
    length = float(spec["system_length"])
    beta = spec["beta"]
    from jellyfysh.base import factory
    from jellyfysh.base.exceptions import EndOfRun
    from jellyfysh.base.node import Node, yield_leaf_nodes
    from jellyfysh.base.particle import Particle
    from jellyfysh.base.strings import to_camel_case
    from jellyfysh.input_output_handler.input_handler.random_node_creator import water_random_node_creator
    from jellyfysh.state_handler.tree_state_handler import TreeStateHandler
    from jellyfysh.scheduler.heap_scheduler.heap_scheduler import HeapScheduler
    import jellyfysh.event_handler.two_leaf_unit_event_handler as m_pair
    import jellyfysh.event_handler.two_composite_object_summed_bounding_potential_event_handler as m_composite
    import jellyfysh.lifting.lifting as m_lifting
    import jellyfysh.event_handler.single_independent_active_periodic_direction_end_of_chain_event_handler as m_eoc

    ctx = {"commits": 0, "target": None, "winner": None, "composite_targets": [], "randint": 0}

    def event_index():
        return ctx["commits"] - 1

    def leaf_index(unit):
        return 3 * unit.identifier[0] + unit.identifier[1]

    class PairRandom:
        @staticmethod
        def expovariate(lambd):
            assert lambd == beta
            return oracle.expovariate(oracle.draw(key, event_index(), oracle.RNG_PAIR, ctx["target"]), lambd)

    class CompositeRandom:
        @staticmethod
        def expovariate(lambd):
            assert lambd == beta
            target = ctx["composite_targets"].pop(0)
            return oracle.expovariate(oracle.draw(key, event_index(), oracle.RNG_COMPOSITE, target), lambd)

        @staticmethod
        def uniform(a, b):
            return a + (b - a) * oracle.uniform(oracle.draw(key, event_index(), oracle.RNG_THIN, 0))

    class LiftRandom:
        @staticmethod
        def uniform(a, b):
            return a + (b - a) * oracle.uniform(oracle.draw(key, event_index(), oracle.RNG_LIFT, 0))

    def eoc_randint(a, b):
        assert a == 0
        which = ctx["randint"]
        ctx["randint"] = (which + 1) % 2
        return oracle.randbelow(oracle.draw(key, event_index(), oracle.RNG_NEW_ACTIVE, which), b + 1)

    # The local factor type map looks the active unit up without the membership test that its non-local variant
    # has (activator/tagger/factor_type_maps.py:324-328 against :337): a local factor type that does not name every
    # unit of a molecule (the H-H bond names the two hydrogens) raises KeyError for the others.  The same test is
    # added here; factor types that name every unit are enumerated exactly as before.
    from jellyfysh.activator.tagger import factor_type_maps as m_maps
    local_map = [cls for cls in vars(m_maps).values()
                 if isinstance(cls, type) and hasattr(cls, "_yield_factor_identifier_local")][0]
    original_local = local_map._yield_factor_identifier_local

    def yield_factor_identifier_local(self, active_identifier):
        if active_identifier[1] in self._map.keys():
            yield from original_local(self, active_identifier)
    local_map._yield_factor_identifier_local = yield_factor_identifier_local

    m_pair.random = PairRandom
    m_composite.random = CompositeRandom
    m_lifting.random = LiftRandom
    m_eoc.randint = eoc_randint

    def leaves_of(in_state):
        return [leaf.value for cnode in in_state for leaf in yield_leaf_nodes(cnode)]

    original_pair = m_pair.TwoLeafUnitEventHandler.send_event_time

    def pair_event_time(self, in_state):
        targets = [u for u in leaves_of(in_state) if u.velocity is None]
        assert len(targets) == 1
        ctx["target"] = leaf_index(targets[0])
        return original_pair(self, in_state)
    m_pair.TwoLeafUnitEventHandler.send_event_time = pair_event_time

    composite_class = m_composite.TwoCompositeObjectSummedBoundingPotentialEventHandler
    original_composite = composite_class.send_event_time

    def composite_event_time(self, in_state):
        units = leaves_of(in_state)
        active = [u for u in units if u.velocity is not None][0]
        ctx["composite_targets"] = sorted(leaf_index(u) for u in units if u.identifier[0] != active.identifier[0])
        result = original_composite(self, in_state)
        assert not ctx["composite_targets"]
        return result
    composite_class.send_event_time = composite_event_time

    queue = list(range(spec["molecules_per_side"] ** 3))

    def fill_root_node(self, node):
        m = queue.pop(0)
        atoms = positions[3 * m:3 * m + 3]
        for t in range(3):
            node.add_child(Node(Particle([float(v) for v in atoms[t]], {"electric_charge": float(charges[3 * m + t])})))
        # the barycentre of the molecule (the oxygen plus the mean of the two O-H bonds, as the reference builds it)
        centre = []
        for d in range(3):
            one = ((atoms[0][d] - atoms[1][d]) + length / 2.0) % length - length / 2.0
            two = ((atoms[2][d] - atoms[1][d]) + length / 2.0) % length - length / 2.0
            centre.append((atoms[1][d] + (one + two) / 3.0) % length)
        node.value = Particle(position=centre)
    water_random_node_creator.WaterRandomNodeCreator.fill_root_node = fill_root_node

    original_succeeding = HeapScheduler.get_succeeding_event

    def get_succeeding_event(self):
        handler = original_succeeding(self)
        ctx["winner"] = handler
        return handler
    HeapScheduler.get_succeeding_event = get_succeeding_event

    log = []
    state = {"active": None}

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
        active_unit = [leaf.value for root in self.extract_active_global_state()
                       for leaf in yield_leaf_nodes(root)][0]
        active = leaf_index(active_unit)
        direction = [i for i, v in enumerate(active_unit.velocity) if v != 0.0][0]
        winner = ctx["winner"]
        moved = state["active"]
        kind = None
        if isinstance(winner, m_pair.TwoLeafUnitEventHandler):  # bonds and Lennard-Jones (factory-named subclasses)
            pair_leaves = winner._leaf_units
            target = [leaf_index(u) for u in pair_leaves if leaf_index(u) != moved][0]
            potential = type(winner._potential).__name__
            kind = oracle.EV_PAIR if potential == "LennardJonesPotential" else oracle.EV_BOND
            accepted = int(active != moved)
        elif isinstance(winner, composite_class):
            kind = oracle.EV_COMPOSITE
            target = winner._target_leaf_units[0].identifier[0]
            accepted = int(active != moved)
        elif isinstance(winner, m_eoc.SingleIndependentActivePeriodicDirectionEndOfChainEventHandler):
            kind = oracle.EV_END_OF_CHAIN
            target = active
            accepted = 1
        if kind is not None:
            moved_branch = self.extract_from_global_state((moved // 3, moved % 3))
            moved_position = [leaf.value for leaf in yield_leaf_nodes(moved_branch)][0].position
            time = winner._event_time
            log.append((kind, moved, target, active, direction, accepted, time.quotient, time.remainder,
                        moved_position[0], moved_position[1], moved_position[2]))
            if len(log) >= spec["events"]:
                raise Stop()
        state["active"] = active
        return result
    TreeStateHandler.insert_into_global_state = insert_into_global_state

    with tempfile.TemporaryDirectory() as scratch:
        factor_file = os.path.join(scratch, "factor_set_water_c5.txt")
        with open(factor_file, "w") as handle:
            handle.write(FACTORS)
        config = configparser.ConfigParser()
        config.read_string(config_text(spec, factor_file))
        factory.build_from_config(config, to_camel_case(config.get("Run", "setting")), "jellyfysh.setting")
        mediator = factory.build_from_config(config, to_camel_case(config.get("Run", "mediator")),
                                             "jellyfysh.mediator")
        try:
            mediator.run()
        except (Stop, EndOfRun):
            pass
    molecules = spec["molecules_per_side"] ** 3
    final = np.array([[leaf.value.position for leaf in
                       yield_leaf_nodes(mediator._state_handler.extract_from_global_state((m, t)))][0]
                      for m in range(molecules) for t in range(3)], dtype=np.float64)
    structured = np.zeros(len(log), dtype=oracle.EVENT_DTYPE)
    for field_index, field in enumerate(oracle.EVENT_DTYPE.names):
        structured[field] = [row[field_index] for row in log]
    out = os.path.join(HERE, "%s.npz" % name)
    np.savez_compressed(out, events=structured, initial=positions, final=final, charges=charges,
                        spec=json.dumps(dict(spec, rng_key=key)))
    print("%s: %d events, kinds %s -> %s" % (name, len(log), np.bincount(structured["kind"], minlength=10), out))


def main(tree, names):
    for name in names:
        subprocess.run([sys.executable, os.path.abspath(__file__), "--one", tree, name], check=True)


if __name__ == "__main__":
    from _tree import tree_argument
    if len(sys.argv) > 1 and sys.argv[1] == "--one":
        run_one(sys.argv[2], sys.argv[3])
    else:
        main(tree_argument(sys.argv), sys.argv[2:] or list(SYSTEMS))
