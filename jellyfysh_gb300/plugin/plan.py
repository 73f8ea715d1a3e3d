"""Translation of a run configured for the reference into a batch of GPU chains, and its execution.

``translate`` reads the system from the objects the reference's factory built (setting, initial units, taggers
with their event handlers and potentials, cell occupancy, far field, chain and run control) into a ``BatchPlan``
(atoms) or a ``WaterPlan`` (water molecules as composite objects with factor-type-map taggers), without running any
of the reference's initialisation (whose far-field tables take minutes in Python); ``run_plan`` executes a plan on
the GPU until the end-of-run time.  Configurations outside the engines' scope (other potentials, taggers or
composite objects) raise ``ConfigurationError``.  Nothing here imports the reference: ``translate`` only reads the
objects it is given.
"""
import dataclasses
import math
from typing import Any, List, Optional

import numpy as np

from jellyfysh_gb300.chains import ChainSpec


class ConfigurationError(Exception):
    """A configured run that the GPU engine does not cover."""


@dataclasses.dataclass
class BatchPlan:
    """One configured system run as `chains` independent chains on the GPU."""
    spec: ChainSpec
    positions: np.ndarray
    charges: Optional[np.ndarray]
    end_of_run_time: float
    chains: int = 1
    mode: str = "mixed"
    seed: int = 0
    events_per_launch: int = 256


def _name(obj) -> str:
    """Class name of a factory-built object; the factory renames aliased classes 'Alias (RealClass)'
    (``base/factory.py:22-60``), whose real class name is the one in parentheses."""
    name = type(obj).__name__
    if name.endswith(")") and "(" in name:
        return name[name.rindex("(") + 1:-1].strip()
    return name


def _potential_kind(potential) -> str:
    name = _name(potential)
    for kind in ("HardSphere", "LennardJones", "MergedImageCoulomb", "InversePowerCoulombBounding"):
        if kind in name:
            return kind
    raise ConfigurationError("potential %s is not on the GPU engine's path" % name)


def _hs_radius(potential) -> float:
    if hasattr(potential, "_radius"):
        return float(potential._radius)
    # the reference keeps 4 r^2 only; sqrt(fl(x^2)) == |x| in IEEE arithmetic, so the radius is recovered exactly
    return math.sqrt(potential._diameter_squared) / 2.0


def _lennard_jones(potential):
    """(prefactor, characteristic length) of the reference's class or of the GPU drop-in."""
    return float(potential._prefactor), float(potential._characteristic_length)


@dataclasses.dataclass
class WaterPlan:
    """One configured water system run as `chains` independent chains on the GPU (``jellyfysh_gb300.water``).  With
    molecular cells (the reference's water cell-veto configuration) ``roots`` holds the root units' positions and
    ``cell_veto`` the cell system and the dipole estimator's parameters, from which ``run_plan`` builds the bound
    tables on the GPU."""
    model: Any
    positions: np.ndarray
    charges: np.ndarray
    end_of_run_time: float
    chains: int = 1
    mode: str = "mixed"
    seed: int = 0
    events_per_launch: int = 256
    roots: Optional[np.ndarray] = None
    cell_veto: Optional[dict] = None


_LIFTINGS = {"InsideFirstLifting": "inside_first", "OutsideFirstLifting": "outside_first",
             "RatioLifting": "ratio"}


def _factor_groups(tagger) -> set:
    """The factors of a factor-type-map tagger as sorted tuples of leaf numbers
    (``activator/tagger/factor_type_maps.py:286-352``)."""
    mapping = tagger._factor_type_map._map
    return {tuple(sorted(group)) for groups in mapping.values() for group in groups}


def _translate_water(state_handler, activator, setting, roots, chains, mode, seed, events_per_launch) -> WaterPlan:
    """Water molecules of three units (hydrogen, oxygen, hydrogen: unit 1 the oxygen) with harmonic O-H and H-H bonds,
    Lennard-Jones between the oxygens and one Coulomb factor per pair of molecules, all through
    ``FactorTypeMapInStateTagger`` (``activator/tagger/factor_type_map_in_state_tagger.py``)."""
    from jellyfysh_gb300.water import WaterModel
    if setting.number_of_nodes_per_root_node != 3 or any(len(node.children) != 3 for node in roots):
        raise ConfigurationError("the water engine runs composite objects of three units")
    roots = sorted(roots, key=lambda node: node.value.identifier)
    leaves = [leaf.value for node in roots for leaf in sorted(node.children, key=lambda c: c.value.identifier)]
    positions = np.array([unit.position for unit in leaves], dtype=np.float64)
    labels = set().union(*[set(unit.charge or {}) for unit in leaves])
    if len(labels) != 1:
        raise ConfigurationError("the water units need exactly one charge: %s" % sorted(labels))
    label = labels.pop()
    charges = np.array([float(unit.charge[label]) for unit in leaves])
    fields = dict(molecules=len(roots), system_length=float(setting.system_length), beta=float(setting.beta),
                  mode=mode)
    bonds = {}
    end_of_run_time = math.inf
    pair_tags, cell_tags, end_of_chain_tags, trash_lists = set(), set(), set(), {}
    boundary_tag, veto, coulomb_taggers = None, None, set()

    def coulomb_factor(handler):
        """The parameters of a summed-bounding Coulomb factor: merged-image Coulomb with the inverse-power bound and
        a lifting scheme."""
        mic, bound = handler._potential, handler._bounding_potential
        if _potential_kind(mic) != "MergedImageCoulomb" or _potential_kind(bound) != "InversePowerCoulombBounding":
            raise ConfigurationError("the Coulomb factor runs merged-image Coulomb with its inverse-power bound")
        fields.update(coulomb_prefactor=float(mic._prefactor), alpha=float(mic._alpha),
                      fourier_cutoff=int(mic._fourier_cutoff), position_cutoff=int(mic._position_cutoff),
                      bound_prefactor=float(bound._prefactor), lifting=lifting_of(handler))

    def lifting_of(handler):
        name = _name(handler._lifting)
        lifting = name.replace("Gpu", "", 1) if name.startswith("Gpu") else name
        if lifting not in _LIFTINGS:
            raise ConfigurationError("lifting scheme %s is not on the water engine's path" % lifting)
        return _LIFTINGS[lifting]

    for tagger in activator._taggers:
        tagger_name = _name(tagger)
        handler = tagger._event_handler_to_copy
        handler_name = _name(handler)
        trash_lists[tagger.tag] = set(tagger.trashes)
        if tagger_name == "CellBoundaryTagger" and handler_name == "CellBoundaryEventHandler":
            boundary_tag = tagger.tag
            cell_tags.add(tagger.tag)
            continue
        if tagger_name in ("ExcludedCellsTagger", "SurplusCellsTagger"):
            if handler_name != "TwoCompositeObjectSummedBoundingPotentialEventHandler":
                raise ConfigurationError("the molecular cells take the summed-bounding Coulomb factor")
            coulomb_factor(handler)
            coulomb_taggers.add(tagger_name)
            cell_tags.add(tagger.tag)
            continue
        if tagger_name == "CellVetoTagger":
            if handler_name != "CompositeObjectCellVetoEventHandler":
                raise ConfigurationError("the water engine's cell veto is the molecular one")
            estimator = handler._estimator
            if _name(estimator) != "DipoleMonteCarloEstimator":
                raise ConfigurationError("the molecular cell veto's bounds come from the dipole Monte Carlo estimator")
            veto = dict(estimator=estimator, lifting=lifting_of(handler), far="cell_veto")
            cell_tags.add(tagger.tag)
            continue
        if tagger_name == "CellBoundingPotentialTagger":
            if handler_name != "TwoCompositeObjectCellBoundingPotentialEventHandler":
                raise ConfigurationError("the water engine's cell-bounding factor is the molecular one")
            mic, bounding = handler._potential, handler._bounding_potential
            estimator = getattr(bounding, "_estimator", None)
            if _name(bounding) != "CellBoundingPotential" or _name(estimator) != "DipoleMonteCarloEstimator":
                raise ConfigurationError("the molecular cell-bounding factor takes the cell-bounding potential of the "
                                         "dipole Monte Carlo estimator")
            if _potential_kind(mic) != "MergedImageCoulomb":
                raise ConfigurationError("the molecular cell-bounding factor bounds merged-image Coulomb")
            veto = dict(estimator=estimator, lifting=lifting_of(handler), far="cell_bounding")
            cell_tags.add(tagger.tag)
            continue
        if tagger_name == "FactorTypeMapInStateTagger":
            pair_tags.add(tagger.tag)
            groups = _factor_groups(tagger)
            if handler_name == "TwoLeafUnitEventHandler":
                potential = handler._potential
                if _name(potential) == "DisplacedEvenPowerPotential":
                    if int(potential._power) != 2:
                        raise ConfigurationError("the water engine's bonds are harmonic (power 2)")
                    for group in groups:
                        if group not in ((0, 1), (1, 2), (0, 2)):
                            raise ConfigurationError("bond factor %s is not within one water molecule" % (group,))
                        bonds[group] = (float(potential._equilibrium_separation), float(potential._prefactor))
                elif _potential_kind(potential) == "LennardJones":
                    if groups != {(1, 4)}:
                        raise ConfigurationError("the water engine's Lennard-Jones acts between the oxygens (1, 4)")
                    fields["lj_prefactor"], fields["lj_sigma"] = _lennard_jones(potential)
                else:
                    raise ConfigurationError("potential %s is not on the water engine's path" % _name(potential))
            elif handler_name == "TwoCompositeObjectSummedBoundingPotentialEventHandler":
                if groups != {(0, 1, 2, 3, 4, 5)}:
                    raise ConfigurationError("the water engine's Coulomb factor takes both molecules whole")
                coulomb_factor(handler)
                pair_tags.discard(tagger.tag)
                coulomb_taggers.add(tagger_name)
            else:
                raise ConfigurationError("factor event handler %s is not on the water engine's path" % handler_name)
        elif handler_name == "SingleIndependentActivePeriodicDirectionEndOfChainEventHandler":
            fields["chain_time"] = float(handler._chain_time)
            end_of_chain_tags.add(tagger.tag)
        elif handler_name == "InitialChainStartOfRunEventHandler":
            velocity = list(handler._initial_velocity)
            direction = [i for i, v in enumerate(velocity) if v != 0.0]
            identifier = tuple(handler._initial_active_identifier)
            if len(direction) != 1 or velocity[direction[0]] <= 0.0 or len(identifier) != 2:
                raise ConfigurationError("the water engine starts one active unit moving along +x, +y or +z")
            fields.update(initial_direction=direction[0], speed=float(velocity[direction[0]]),
                          initial_active=3 * int(identifier[0]) + int(identifier[1]))
        elif handler_name == "FinalTimeEndOfRunEventHandler":
            end_of_run_time = float(handler._event_time.quotient + handler._event_time.remainder)
        else:
            raise ConfigurationError("tagger %s with %s is not on the water engine's path" % (tagger_name,
                                                                                           handler_name))
    if set(bonds) != {(0, 1), (1, 2), (0, 2)} or bonds[(0, 1)] != bonds[(1, 2)]:
        raise ConfigurationError("the water engine needs the two O-H bonds (alike) and the H-H bond")
    fields["oh_r0"], fields["oh_prefactor"] = bonds[(0, 1)]
    fields["hh_r0"], fields["hh_prefactor"] = bonds[(0, 2)]
    for key in ("chain_time", "initial_direction", "lj_prefactor", "coulomb_prefactor"):
        if key not in fields:
            raise ConfigurationError("the water system lacks %s" % key)
    cell_veto, root_positions = None, None
    if cell_tags:
        cell_veto = _water_cells(activator, fields, coulomb_taggers, boundary_tag, veto, pair_tags, cell_tags,
                                 end_of_chain_tags, trash_lists)
        root_positions = np.array([node.value.position for node in roots], dtype=np.float64)
    return WaterPlan(model=WaterModel(**fields), positions=positions, charges=charges,
                     end_of_run_time=end_of_run_time, chains=int(chains), mode=mode, seed=int(seed),
                     events_per_launch=int(events_per_launch), roots=root_positions, cell_veto=cell_veto)


def _water_cells(activator, fields, coulomb_taggers, boundary_tag, veto, pair_tags, cell_tags, end_of_chain_tags,
                 trash_lists) -> dict:
    """The molecular cells of a water configuration as the reference's water cell-veto configuration sets them up
    (``config_files/2018_JCP_149_064113/water/coulomb_cell_veto_lj_inverted.ini``): one single-active cell
    occupancy of the root units on cubic periodic cells, the nearby and surplus Coulomb factors, the molecular cell
    veto with the dipole Monte Carlo estimator (or the molecular cell-bounding factor on it, as
    ``config_files/2018_JCP_149_064113/dipoles/cell_bounded.ini`` sets it up), and the cell boundary; every other event
    recreates every factor."""
    if coulomb_taggers != {"ExcludedCellsTagger", "SurplusCellsTagger"} or boundary_tag is None or veto is None:
        raise ConfigurationError("the molecular cells need the nearby and surplus Coulomb factors, the cell veto or "
                                 "the cell-bounding factor, and the cell boundary")
    occupancies = [s for s in activator._internal_states if _name(s) == "SingleActiveCellOccupancy"]
    if len(occupancies) != 1 or int(occupancies[0]._cell_level) != 1:
        raise ConfigurationError("the molecular cells need one single-active cell occupancy of the root units")
    occupancy = occupancies[0]
    cells = occupancy._cells
    if _name(cells) != "CuboidPeriodicCells" or len(set(cells._cells_per_side)) != 1:
        raise ConfigurationError("the water engine needs cubic periodic cells")
    if int(occupancy._maximum_number_occupants) != 1:
        raise ConfigurationError("the molecular cells hold one occupant per cell")
    if veto["lifting"] != fields["lifting"]:
        raise ConfigurationError("the far field and the Coulomb factors lift with the same scheme")
    estimator = veto["estimator"]
    mic = estimator._potential
    if _potential_kind(mic) != "MergedImageCoulomb" or (
            float(mic._prefactor), float(mic._alpha), int(mic._fourier_cutoff), int(mic._position_cutoff)) != (
            fields["coulomb_prefactor"], fields["alpha"], fields["fourier_cutoff"], fields["position_cutoff"]):
        raise ConfigurationError("the dipole estimator bounds the Coulomb factors' merged-image potential")
    everything = pair_tags | cell_tags
    for tag, trashed in trash_lists.items():
        if tag != boundary_tag and tag in everything | end_of_chain_tags and not everything <= trashed:
            raise ConfigurationError("tagger %s must trash every pair and cell factor" % tag)
    boundary_trash = trash_lists[boundary_tag] & everything
    if boundary_trash == everything:
        keep_pairs = False
    elif boundary_trash == cell_tags:
        keep_pairs = True
    else:
        raise ConfigurationError("the cell boundary trashes the cell factors, with or without the pair factors")
    return dict(cells_per_side=int(cells._cells_per_side[0]), neighbor_layers=int(cells._neighbor_layers),
                dipole_separation=float(estimator._dipole_separation), dipole_charge=float(estimator._dipole_charge),
                prefactor=float(estimator._prefactor), number_trials=int(estimator._number_trials),
                empirical_bound=float(estimator._empirical_bound), keep_pairs=keep_pairs, far=veto["far"])


def translate(state_handler, activator, setting, chains: int = 1, mode: str = "mixed", seed: int = 0,
              events_per_launch: int = 256):
    """Read a configured run from the reference's constructed objects (the hypercubic setting module
    ``setting/hypercubic_setting.py``, taggers ``activator/tagger/*.py``, event
    handlers ``event_handler/*.py``, potentials ``potential/*.py``, occupancy
    ``activator/internal_state/single_active_cell_occupancy.py``, cells
    ``activator/internal_state/cell_occupancy/cells/cuboid_periodic_cells.py``)."""
    if not setting.initialized() or setting.dimension != 3:
        raise ConfigurationError("the GPU engine runs three-dimensional hypercubic settings")
    length = float(setting.system_length)
    beta = float(setting.beta)
    roots = state_handler.extract_global_state()
    if any(node.children for node in roots):
        return _translate_water(state_handler, activator, setting, roots, chains, mode, seed, events_per_launch)
    roots = sorted(roots, key=lambda node: node.value.identifier)
    positions = np.array([node.value.position for node in roots], dtype=np.float64)
    n = len(roots)

    occupancies = [s for s in activator._internal_states if _name(s) == "SingleActiveCellOccupancy"]
    if len(occupancies) != 1:
        raise ConfigurationError("the GPU engine needs one single-active cell occupancy")
    occupancy = occupancies[0]
    cells = occupancy._cells
    if _name(cells) != "CuboidPeriodicCells" or len(set(cells._cells_per_side)) != 1:
        raise ConfigurationError("the GPU engine needs cubic periodic cells")
    max_occupants = int(occupancy._maximum_number_occupants)

    fields = dict(n=n, system_length=length, cells_per_side=int(cells._cells_per_side[0]),
                  neighbor_layers=int(cells._neighbor_layers), max_occupants=max(max_occupants, 1), beta=beta)
    pair_potentials: List[Any] = []
    bounded = None
    far = "none"
    estimator = None
    charge_label = None
    end_of_run_time = math.inf
    for tagger in activator._taggers:
        tagger_name = _name(tagger)
        handler = tagger._event_handler_to_copy
        handler_name = _name(handler)
        if tagger_name in ("ExcludedCellsTagger", "SurplusCellsTagger"):
            if handler_name == "TwoLeafUnitEventHandler":
                pair_potentials.append(handler._potential)
            elif handler_name == "TwoLeafUnitBoundingPotentialEventHandler":
                bounded = handler
            else:
                raise ConfigurationError("pair event handler %s is not on the GPU engine's path" % handler_name)
        elif tagger_name == "CellBoundingPotentialTagger":
            far = "cell_bounding"
            estimator = handler._bounding_potential._estimator
        elif tagger_name == "CellVetoTagger":
            far = "cell_veto"
            estimator = handler._estimator
            charge_label = getattr(handler, "_charge", None) or charge_label
        elif handler_name == "CellBoundaryEventHandler":
            pass
        elif handler_name == "SingleIndependentActivePeriodicDirectionEndOfChainEventHandler":
            fields["chain_time"] = float(handler._chain_time)
        elif handler_name == "InitialChainStartOfRunEventHandler":
            velocity = list(handler._initial_velocity)
            direction = [i for i, v in enumerate(velocity) if v != 0.0]
            if len(direction) != 1 or velocity[direction[0]] <= 0.0 or len(handler._initial_active_identifier) != 1:
                raise ConfigurationError("the GPU engine starts one active unit moving along +x, +y or +z")
            fields.update(initial_direction=direction[0], speed=float(velocity[direction[0]]),
                          initial_active=int(handler._initial_active_identifier[0]))
        elif handler_name == "FinalTimeEndOfRunEventHandler":
            end_of_run_time = float(handler._event_time.quotient + handler._event_time.remainder)
        else:
            raise ConfigurationError("tagger %s with %s is not on the GPU engine's path" % (tagger_name,
                                                                                         handler_name))
    if "chain_time" not in fields or "initial_direction" not in fields:
        raise ConfigurationError("the GPU engine needs the end-of-chain and start-of-run handlers of the path")

    charges = None
    kinds = sorted({_potential_kind(p) for p in pair_potentials})
    if bounded is not None:
        if _potential_kind(bounded._potential) != "MergedImageCoulomb" or \
                _potential_kind(bounded._bounding_potential) != "InversePowerCoulombBounding":
            raise ConfigurationError("bounded pair events run merged-image Coulomb with its inverse-power bound")
        mic = bounded._potential
        fields.update(potential="coulomb", coulomb_prefactor=float(mic._prefactor), ewald_alpha=float(mic._alpha),
                      fourier_cutoff=int(mic._fourier_cutoff), position_cutoff=int(mic._position_cutoff),
                      bound_prefactor=float(bounded._bounding_potential._prefactor))
        if kinds == ["HardSphere"]:
            fields["hs_radius"] = _hs_radius(pair_potentials[0])
        elif kinds:
            raise ConfigurationError("a Coulomb system takes a hard core as its only other pair potential")
        # the charge label of the handlers: a cell-veto handler keeps it; else the units' only charge
        labels = set().union(*[set(node.value.charge or {}) for node in roots])
        label = charge_label or (labels.pop() if len(labels) == 1 else None)
        if label is None:
            raise ConfigurationError("the units' charge for the Coulomb handlers is ambiguous: %s" % sorted(labels))
        charges = np.array([float(node.value.charge[label]) for node in roots])
    elif kinds == ["HardSphere"]:
        fields.update(potential="hard_sphere", hs_radius=_hs_radius(pair_potentials[0]))
    elif kinds == ["LennardJones"]:
        prefactor, sigma = _lennard_jones(pair_potentials[0])
        fields.update(potential="lennard_jones", lj_prefactor=prefactor, lj_sigma=sigma)
    else:
        raise ConfigurationError("pair potentials %s are not one potential of the GPU engine's path" % kinds)
    fields["far"] = far
    if estimator is not None:
        if _name(estimator) != "InnerPointEstimator":
            raise ConfigurationError("the GPU engine bounds the far field with the inner-point estimator")
        fields.update(estimator_points=int(estimator._points_per_side),
                      estimator_prefactor=float(estimator._prefactor))
    if far != "none" and fields["max_occupants"] != 1:
        raise ConfigurationError("the far fields need at most one occupant per cell")
    spec = ChainSpec(**fields)
    return BatchPlan(spec=spec, positions=positions, charges=charges, end_of_run_time=end_of_run_time,
                     chains=int(chains), mode=mode, seed=int(seed), events_per_launch=int(events_per_launch))


def run_plan(plan, stop_time: Optional[float] = None, device: str = "cuda:0"):
    """Advance every chain of the plan to `stop_time` (default: the end-of-run time); returns the ChainBatch or
    WaterBatch."""
    from jellyfysh_gb300 import ChainBatch
    t_stop = plan.end_of_run_time if stop_time is None else float(stop_time)
    if math.isinf(t_stop):
        raise ConfigurationError("the run needs a finite end-of-run time")
    if isinstance(plan, WaterPlan):
        import torch
        from jellyfysh_gb300.water import WaterBatch
        with torch.cuda.device(torch.device(device)):
            cells, roots = None, None
            if plan.cell_veto is not None:
                from jellyfysh_gb300.water import dipole_cell_veto_bounds
                cells = dipole_cell_veto_bounds(plan.model, seed=plan.seed, **plan.cell_veto)
                roots = np.repeat(plan.roots[None], plan.chains, axis=0)
            batch = WaterBatch(plan.model, np.repeat(plan.positions[None], plan.chains, axis=0), seed=plan.seed,
                               charges=plan.charges, cells=cells, roots=roots)
            while True:
                batch.run(plan.events_per_launch, stop_time=t_stop)
                batch.check_status()
                if (batch.states()["stopped"] == 1).all():
                    return batch
    charges = None if plan.charges is None else [plan.charges] * plan.chains
    batch = ChainBatch([plan.spec] * plan.chains, [plan.positions] * plan.chains, charges, seed=plan.seed,
                       device=device)
    while True:
        batch.run(plan.events_per_launch, stop_time=t_stop, mode=plan.mode)
        batch.check_status()
        state = batch.state()
        reached = state["stopped"] == 1
        if reached.all():
            return batch
