"""Record event-by-event trajectories of the reference's event loop for flexible water with the molecular cell veto.

Run in a container that holds the JeLLyFysh source tree with its cffi extensions built:

    python tests/golden/make_water_cell_trajectories.py /path/to/jellyfysh/tree [name ...]

The water model is the one of ``make_water_trajectories.py`` (harmonic O–H and H–H bonds, Lennard-Jones between
oxygens through the factor-type-map tagger, merged-image Coulomb between molecules, inside-first lifting, periodic
direction end of chain).  The Coulomb interaction between molecules is set up as in the reference's water cell-veto
configuration (``config_files/2018_JCP_149_064113/water/coulomb_cell_veto_lj_inverted.ini``):

* ``SingleActiveCellOccupancy`` of the molecules (``cell_level = 1``: the root units, at the molecules' barycentres)
  on ``CuboidPeriodicCells`` with two neighbour layers;
* ``molecule_cell_boundary`` (``CellBoundaryEventHandler`` on the active root unit, which moves at a third of the
  active leaf unit's velocity); it trashes and creates only the cell-based factors, so that the bond and
  Lennard-Jones candidates persist across it;
* ``coulomb_nearby`` (``ExcludedCellsTagger``) and ``coulomb_surplus`` (``SurplusCellsTagger``):
  ``TwoCompositeObjectSummedBoundingPotentialEventHandler`` against the molecules of the nearby cells and the surplus
  molecules;
* ``coulomb_cell_veto`` (``CellVetoTagger``): ``CompositeObjectCellVetoEventHandler`` with the
  ``DipoleMonteCarloEstimator`` of the reference configuration (dipole separation 0.5, dipole charge 0.82, prefactor
  1.5, 1000 trials, empirical bound 30).

Two trajectories take the molecular cell-bounding far field instead of the cell veto
(``CellBoundingPotentialTagger`` with ``TwoCompositeObjectCellBoundingPotentialEventHandler`` and a
``CellBoundingPotential`` on the same estimator, as the reference's dipole configuration
``config_files/2018_JCP_149_064113/dipoles/cell_bounded.ini`` sets it up): one candidate per occupied far cell, whose
potential change is keyed by the target molecule (kind RNG_CELL_BOUND).

The bending potential of the reference configuration is not part of the model (it is not one of the factors of the
event-time path this project rebuilds).  As for the other trajectories, the initial state, the random numbers of the
event loop (keyed draws of the oracle's generator: pair changes by target unit, Coulomb factor changes by target
unit, thinning, lifting, the cell veto's Walker choice, Walker uniform and time, the end of chain's integers) and the
output are replaced around the unchanged ``SingleProcessMediator.run``; the estimator draws from Python's ``random``,
seeded, and its bound tables are stored with the trajectory.  Every committed event is logged with the position of
the moved leaf unit and of its molecule's root unit.
"""
import json
import os
import random
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
from make_water_trajectories import FACTORS, WATER, initial_state  # noqa: E402

CELL_VETO = dict(cells_per_side=8, neighbor_layers=2, dipole_separation=0.5, dipole_charge=0.82,
                 estimator_prefactor=1.5, number_trials=1000, empirical_bound=30.0)
SYSTEMS = {
    # the batched water of the benchmark: 64 molecules, 8^3 cells, two neighbour layers
    "water_n64_cell_veto": dict(WATER, **CELL_VETO, molecules_per_side=4, system_length=12.42, seed=24,
                                events=12000),
    # 8 molecules, 4^3 cells and one neighbour layer (the far field holds 37 of the 64 cells), the estimator's
    # empirical bound lowered to 2 so that the far field's events leave room for many cell-boundary events (the
    # bound does not bound every rate then: the reference only warns, and the trajectory stays a trajectory of its
    # event loop)
    "water_n8_cell_veto": dict(WATER, **dict(CELL_VETO, cells_per_side=4, neighbor_layers=1, empirical_bound=2.0),
                               molecules_per_side=2, system_length=12.42 / 2.0, seed=25, events=5000),
    # 8 molecules, 6^3 cells of 1.035 and one neighbour layer, the far field nearly off (empirical bound 0.02): the
    # root units cross many cell boundaries, and the bond and Lennard-Jones candidates that persist across them often
    # come next, committing the in-state copies of their creation
    "water_n8_cell_boundaries": dict(WATER, **dict(CELL_VETO, cells_per_side=6, neighbor_layers=1,
                                                   empirical_bound=0.02),
                                     molecules_per_side=2, system_length=12.42 / 2.0, seed=26, events=5000),
    # the molecular cell-bounding far field instead of the cell veto
    # (TwoCompositeObjectCellBoundingPotentialEventHandler with CellBoundingPotentialTagger, as the reference's dipole
    # configuration config_files/2018_JCP_149_064113/dipoles/cell_bounded.ini sets it up): one candidate per occupied
    # far cell; 8 molecules on 4^3 cells with one neighbour layer, and 64 molecules on 6^3 cells with one layer
    "water_n8_cell_bounding": dict(WATER, **dict(CELL_VETO, cells_per_side=4, neighbor_layers=1, empirical_bound=2.0),
                                   far="cell_bounding", molecules_per_side=2, system_length=12.42 / 2.0, seed=27,
                                   events=4000),
    "water_n64_cell_bounding": dict(WATER, **dict(CELL_VETO, cells_per_side=6, neighbor_layers=1,
                                                  empirical_bound=5.0),
                                    far="cell_bounding", molecules_per_side=4, system_length=12.42, seed=28,
                                    events=2500),
}

PAIR_TAGS = ["harmonic_oh", "harmonic_hh", "lennard_jones"]
CELL_TAGS = ["molecule_cell_boundary", "coulomb_nearby", "coulomb_surplus", "coulomb_cell_veto"]
FAR_TAGGERS = {"cell_veto": "coulomb_cell_veto (cell_veto_tagger)",
               "cell_bounding": "coulomb_cell_bounding (cell_bounding_potential_tagger)"}


def cell_tags(spec):
    return [t if t != "coulomb_cell_veto" or spec.get("far", "cell_veto") == "cell_veto" else "coulomb_cell_bounding"
            for t in CELL_TAGS]


def far_sections(spec, every):
    molecules = spec["molecules_per_side"] ** 3
    if spec.get("far", "cell_veto") == "cell_veto":
        return """[CoulombCellVeto]
trash = {every}
create = {every}
event_handler = coulomb_cell_veto_event_handler (composite_object_cell_veto_event_handler)
internal_state_label = single_active_cell_occupancy

[CoulombCellVetoEventHandler]
estimator = dipole_monte_carlo_estimator
lifting = inside_first_lifting
charge = electric_charge
""".format(every=every)
    return """[CoulombCellBounding]
trash = {every}
create = {every}
event_handler = two_composite_object_cell_bounding_potential_event_handler
internal_state_label = single_active_cell_occupancy
number_event_handlers = {others}

[TwoCompositeObjectCellBoundingPotentialEventHandler]
potential = merged_image_coulomb_potential
bounding_potential = cell_bounding_potential
lifting = inside_first_lifting
charge = electric_charge

[CellBoundingPotential]
estimator = dipole_monte_carlo_estimator
""".format(every=every, others=molecules - 1)


def config_text(spec, factor_file):
    molecules = spec["molecules_per_side"] ** 3
    tags = cell_tags(spec)
    every = ", ".join(PAIR_TAGS + tags)
    cells = ", ".join(tags)
    sections = []
    pair_handlers = {"harmonic_oh": ("harmonic_oh_event_handler (two_leaf_unit_event_handler)", 2),
                     "harmonic_hh": ("harmonic_hh_event_handler (two_leaf_unit_event_handler)", 1),
                     "lennard_jones": ("lennard_jones_event_handler (two_leaf_unit_event_handler)", molecules - 1)}
    for tag in PAIR_TAGS:
        handler, count = pair_handlers[tag]
        sections.append("[%s]\ncreate = %s\ntrash = %s\nevent_handler = %s\nnumber_event_handlers = %d\n"
                        "factor_type_maps = factor_type_maps\n" % (
                            "".join(p.capitalize() for p in tag.split("_")), every, every, handler, count))
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
    molecule_cell_boundary (cell_boundary_tagger),
    coulomb_nearby (excluded_cells_tagger),
    coulomb_surplus (surplus_cells_tagger),
    {far_tagger},
    end_of_chain (active_global_state_in_state_tagger),
    end_of_run (no_in_state_tagger),
    start_of_run (no_in_state_tagger)
internal_states = single_active_cell_occupancy

[SingleActiveCellOccupancy]
cells = cuboid_periodic_cells
cell_level = 1

[CuboidPeriodicCells]
cells_per_side = {m}, {m}, {m}
neighbor_layers = {layers}

[FactorTypeMaps]
filename = {factor_file}

{sections}
[MoleculeCellBoundary]
trash = {cells}
create = {cells}
internal_state_label = single_active_cell_occupancy
event_handler = cell_boundary_event_handler

[CoulombNearby]
trash = {every}
create = {every}
event_handler = coulomb_exception_event_handler (two_composite_object_summed_bounding_potential_event_handler)
internal_state_label = single_active_cell_occupancy
number_event_handlers = {others}

[CoulombSurplus]
trash = {every}
create = {every}
event_handler = coulomb_exception_event_handler (two_composite_object_summed_bounding_potential_event_handler)
internal_state_label = single_active_cell_occupancy
number_event_handlers = {others}

{far_sections}
[CoulombExceptionEventHandler]
potential = merged_image_coulomb_potential
bounding_potential = inverse_power_coulomb_bounding_potential
lifting = inside_first_lifting
charge = electric_charge

[MergedImageCoulombPotential]
prefactor = {coulomb_prefactor!r}
alpha = {alpha!r}
fourier_cutoff = {fourier_cutoff}
position_cutoff = {position_cutoff}

[InversePowerCoulombBoundingPotential]
prefactor = {bound_prefactor!r}

[DipoleMonteCarloEstimator]
potential = merged_image_coulomb_potential
dipole_separation = {dipole_separation!r}
dipole_charge = {dipole_charge!r}
prefactor = {estimator_prefactor!r}
number_trials = {number_trials}
empirical_bound = {empirical_bound!r}

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

[EndOfChain]
create = end_of_chain, {every}
trash = end_of_chain, {every}
event_handler = single_independent_active_periodic_direction_end_of_chain_event_handler

[SingleIndependentActivePeriodicDirectionEndOfChainEventHandler]
chain_time = {chain_time!r}

[EndOfRun]
create = end_of_run
trash = end_of_chain, {every}, end_of_run
event_handler = final_time_end_of_run_event_handler

[FinalTimeEndOfRunEventHandler]
end_of_run_time = 1e9

[StartOfRun]
trash = start_of_run
create = end_of_chain, {every}, end_of_run
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
""".format(L=float(spec["system_length"]), factor_file=factor_file, sections="\n".join(sections), every=every,
           cells=cells, m=spec["cells_per_side"], layers=spec["neighbor_layers"], molecules=molecules,
           others=molecules - 1, far_tagger=FAR_TAGGERS[spec.get("far", "cell_veto")],
           far_sections=far_sections(spec, every), **{k: v for k, v in spec.items() if k not in ("lifting", "far")})


def barycentres(positions, length):
    """The root unit of every molecule: the oxygen plus the mean of the two O-H bonds (minimum image), wrapped, in
    Python floats (the arithmetic of ``jellyfysh_gb300.systems.water_roots``)."""
    sys.path.insert(0, ROOT)
    from jellyfysh_gb300 import systems
    return systems.water_roots(positions, length)


def run_one(tree, name):
    spec = SYSTEMS[name]
    sys.path.insert(0, tree)
    sys.path.insert(0, ROOT)
    import configparser
    import logging
    logging.disable(logging.ERROR)
    import oracle
    positions, charges = initial_state(spec)
    length = float(spec["system_length"])
    roots = barycentres(positions, length)
    key = oracle.chain_key(spec["seed"], 0)
    beta = spec["beta"]
    m_cells = spec["cells_per_side"]
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
    import jellyfysh.event_handler.composite_object_cell_veto_event_handler as m_composite_veto
    import jellyfysh.event_handler.two_composite_object_cell_bounding_potential_event_handler as m_cell_bounding
    from jellyfysh.potential.cell_bounding_potential import CellBoundingPotential
    import jellyfysh.event_handler.abstracts.cell_veto_event_handler as m_veto
    import jellyfysh.event_handler.cell_boundary_event_handler as m_boundary
    import jellyfysh.event_handler.walker as m_walker
    import jellyfysh.lifting.lifting as m_lifting
    import jellyfysh.event_handler.single_independent_active_periodic_direction_end_of_chain_event_handler as m_eoc

    ctx = {"commits": 0, "target": None, "winner": None, "composite_targets": [], "randint": 0, "bounds": None}

    def event_index():
        return ctx["commits"] - 1

    def leaf_index(unit):
        return 3 * unit.identifier[0] + unit.identifier[1]

    def cell_index(cell):
        """The flat index of a cuboid cell: its identifier (x, y, z) with x running fastest."""
        return cell.identifier[0] + m_cells * (cell.identifier[1] + m_cells * cell.identifier[2])

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
            return a + (b - a) * oracle.uniform(oracle.draw(key, event_index(), oracle.RNG_VETO_UNIFORM, 0))

    def eoc_randint(a, b):
        assert a == 0
        which = ctx["randint"]
        ctx["randint"] = (which + 1) % 2
        return oracle.randbelow(oracle.draw(key, event_index(), oracle.RNG_NEW_ACTIVE, which), b + 1)

    # the local factor type map's membership test, amended as for the all-pairs water trajectories
    from jellyfysh.activator.tagger import factor_type_maps as m_maps
    local_map = [cls for cls in vars(m_maps).values()
                 if isinstance(cls, type) and hasattr(cls, "_yield_factor_identifier_local")][0]
    original_local = local_map._yield_factor_identifier_local

    def yield_factor_identifier_local(self, active_identifier):
        if active_identifier[1] in self._map.keys():
            yield from original_local(self, active_identifier)
    local_map._yield_factor_identifier_local = yield_factor_identifier_local

    class CellBoundRandom:
        @staticmethod
        def expovariate(lambd):
            assert lambd == beta
            return oracle.expovariate(oracle.draw(key, event_index(), oracle.RNG_CELL_BOUND, ctx["cb_target"]),
                                      lambd)

        @staticmethod
        def uniform(a, b):
            return a + (b - a) * oracle.uniform(oracle.draw(key, event_index(), oracle.RNG_THIN, 0))

    m_pair.random = PairRandom
    m_composite.random = CompositeRandom
    m_composite_veto.random = CompositeRandom
    m_cell_bounding.random = CellBoundRandom
    m_veto.random = VetoRandom
    m_walker.random = WalkerRandom
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

    bounding_class = m_cell_bounding.TwoCompositeObjectCellBoundingPotentialEventHandler
    original_bounding_time = bounding_class.send_event_time

    def bounding_event_time(self, in_state):
        ctx["cb_target"] = in_state[1].value.identifier[0]
        return original_bounding_time(self, in_state)
    bounding_class.send_event_time = bounding_event_time

    original_cell_bounding_initialize = CellBoundingPotential.initialize

    def cell_bounding_initialize(self, cells, calculate_lower_bound):
        original_cell_bounding_initialize(self, cells, calculate_lower_bound)
        if ctx["bounds"] is None:
            ncells = m_cells ** 3
            upper = np.full((ncells, 3), np.nan)
            lower = np.full((ncells, 3), np.nan)
            for cell, values in self._derivative_bounds[0].items():
                upper[cell_index(cell)] = values
            for cell, values in self._derivative_bounds[1].items():
                lower[cell_index(cell)] = [-v for v in values]  # stored negated, as the cell veto stores it
            ctx["bounds"] = (upper, lower)
    CellBoundingPotential.initialize = cell_bounding_initialize

    veto_class = m_composite_veto.CompositeObjectCellVetoEventHandler
    original_initialize = veto_class.initialize

    def initialize(self, cells, cell_level):
        original_initialize(self, cells, cell_level)
        if ctx["bounds"] is None:
            ncells = m_cells ** 3
            upper = np.full((ncells, 3), np.nan)
            lower = np.full((ncells, 3), np.nan)
            for cell, values in self._derivative_bounds.items():
                for d in range(3):
                    upper[cell_index(cell), d] = values[d][0]
                    lower[cell_index(cell), d] = values[d][1]
            ctx["bounds"] = (upper, lower)
    veto_class.initialize = initialize

    queue = list(range(spec["molecules_per_side"] ** 3))

    def fill_root_node(self, node):
        m = queue.pop(0)
        atoms = positions[3 * m:3 * m + 3]
        for t in range(3):
            node.add_child(Node(Particle([float(v) for v in atoms[t]], {"electric_charge": float(charges[3 * m + t])})))
        node.value = Particle(position=[float(v) for v in roots[m]])
    water_random_node_creator.WaterRandomNodeCreator.fill_root_node = fill_root_node

    original_succeeding = HeapScheduler.get_succeeding_event

    def get_succeeding_event(self):
        handler = original_succeeding(self)
        ctx["winner"] = handler
        return handler
    HeapScheduler.get_succeeding_event = get_succeeding_event

    log, root_log = [], []
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
        if isinstance(winner, m_pair.TwoLeafUnitEventHandler):
            target = [leaf_index(u) for u in winner._leaf_units if leaf_index(u) != moved][0]
            kind = oracle.EV_PAIR if type(winner._potential).__name__ == "LennardJonesPotential" else oracle.EV_BOND
            accepted = int(active != moved)
        elif isinstance(winner, composite_class):
            kind = oracle.EV_COMPOSITE
            target = winner._target_leaf_units[0].identifier[0]
            accepted = int(active != moved)
        elif isinstance(winner, bounding_class):
            kind = oracle.EV_CELL_BOUNDING
            target = winner._target_leaf_units[0].identifier[0]
            accepted = int(active != moved)
        elif isinstance(winner, veto_class):
            kind = oracle.EV_CELL_VETO
            target = winner._target_leaf_units[0].identifier[0] if len(winner._state) == 2 else -1
            accepted = int(active != moved)
        elif isinstance(winner, m_boundary.CellBoundaryEventHandler):
            kind = oracle.EV_BOUNDARY
            target = -1
            accepted = 0
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
            root_log.append(list(moved_branch.value.position))
            if len(log) >= spec["events"]:
                raise Stop()
        state["active"] = active
        return result
    TreeStateHandler.insert_into_global_state = insert_into_global_state

    random.seed(spec["seed"])  # the estimator's Monte Carlo trials
    with tempfile.TemporaryDirectory() as scratch:
        factor_file = os.path.join(scratch, "factor_set_water_c5.txt")
        with open(factor_file, "w") as handle:
            handle.write(FACTORS.replace("[0, 1, 2, 3, 4, 5], Coulomb\n", ""))
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
    final_roots = np.array([mediator._state_handler.extract_from_global_state((m, 0)).value.position
                            for m in range(molecules)], dtype=np.float64)
    structured = np.zeros(len(log), dtype=oracle.EVENT_DTYPE)
    for field_index, field in enumerate(oracle.EVENT_DTYPE.names):
        structured[field] = [row[field_index] for row in log]
    upper, lower = ctx["bounds"]
    out = os.path.join(HERE, "%s.npz" % name)
    np.savez_compressed(out, events=structured, roots=np.array(root_log, dtype=np.float64), initial=positions,
                        initial_roots=np.array(roots, dtype=np.float64), final=final, final_roots=final_roots,
                        charges=charges, bounds_upper=upper, bounds_lower=lower,
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
