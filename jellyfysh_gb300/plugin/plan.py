"""Translation of a run configured for the reference into a batch of GPU chains, and its execution.

``translate`` reads the system from the objects the reference's factory built (setting, initial units, taggers
with their event handlers and potentials, cell occupancy, far field, chain and run control) into a ``BatchPlan``,
without running any of the reference's initialisation (whose far-field tables take minutes in Python);
``run_plan`` executes a plan on the GPU until the end-of-run time.  Configurations outside the engine's scope
(composite objects, other potentials or taggers) raise ``ConfigurationError``.  Nothing here imports the
reference: ``translate`` only reads the objects it is given.
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


def translate(state_handler, activator, setting, chains: int = 1, mode: str = "mixed", seed: int = 0,
              events_per_launch: int = 256) -> BatchPlan:
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
    for node in roots:
        if node.children:
            raise ConfigurationError("composite objects are not on the GPU engine's path")
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


def run_plan(plan: BatchPlan, stop_time: Optional[float] = None, device: str = "cuda:0"):
    """Advance every chain of the plan to `stop_time` (default: the end-of-run time); returns the ChainBatch."""
    from jellyfysh_gb300 import ChainBatch
    t_stop = plan.end_of_run_time if stop_time is None else float(stop_time)
    if math.isinf(t_stop):
        raise ConfigurationError("the run needs a finite end-of-run time")
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
