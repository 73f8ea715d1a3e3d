"""GPU drop-in for the pair event handlers of an active unit's neighbourhood.

The reference gives every (active, target) pair of the nearby cells and of the surplus its own
``TwoLeafUnitEventHandler`` (``event_handler/two_leaf_unit_event_handler.py:98-154``, created by
``activator/tagger/excluded_cells_tagger.py:107-132`` and ``surplus_cells_tagger.py:107-131``): one Python solve and
one heap entry per target and event.  ``GpuNeighbourhoodEventHandler`` takes the whole neighbourhood as one in-state
(the active unit and every target, as ``gpu_neighbourhood_tagger`` yields it, in the way the reference's
``cell_bounding_potential_tagger.py:150-155`` yields variable-length in-states) and solves all pairs in one batched
GPU launch of the potential (``displacements`` of the GPU potentials); the earliest pair is its candidate event.
``send_out_state`` is the reference's velocity exchange with that target (``abstracts.py:283-321``).  The events,
their times and the out-states are those of the reference's pair handlers: the earliest of the pair candidates is
what the reference's heap would pop among them.

Configuration (the reference's vocabulary, only the pair taggers change):

    [TagActivator]
    taggers = pair_neighbourhood (gpu_neighbourhood_tagger), ...

    [PairNeighbourhood]
    create = pair_neighbourhood, ...
    trash = pair_neighbourhood, ...
    event_handler = gpu_neighbourhood_event_handler
    internal_state_label = single_active_cell_occupancy

    [GpuNeighbourhoodEventHandler]
    potential = gpu_lennard_jones_potential
"""
import logging
import random
from typing import Sequence

from jellyfysh.base.exceptions import ConfigurationError
from jellyfysh.base.logging import log_init_arguments
from jellyfysh.base.node import Node
from jellyfysh.base.time import Time
from jellyfysh.event_handler.abstracts import SingleActiveLeafUnitEventHandler
from jellyfysh.potential import InvertiblePotential
import jellyfysh.setting as setting

from jellyfysh_gb300.plugin.potential._common import earliest


class GpuNeighbourhoodEventHandler(SingleActiveLeafUnitEventHandler):
    """The earliest pair event of the single active leaf unit against every other leaf unit of the in-state, with a
    GPU potential that solves all pairs in one launch.

    As in the reference's TwoLeafUnitEventHandler, the separations are corrected for the periodic boundaries, the
    charges named by ``charge`` are passed to the potential, and a potential change ``random.expovariate(beta)`` is
    drawn for every pair (one per target, in the in-state's order) when the potential requires one.
    """

    def __init__(self, potential: InvertiblePotential, charge: str = None) -> None:
        log_init_arguments(logging.getLogger(__name__).debug, self.__class__.__name__,
                           potential=potential.__class__.__name__, charge=charge)
        super().__init__()
        if not hasattr(potential, "displacements"):
            raise ConfigurationError("The event handler {0} expects a GPU potential with batched displacements "
                                     "(gpu_..._potential).".format(self.__class__.__name__))
        if potential.number_separation_arguments != 1:
            raise ConfigurationError("The event handler {0} expects a potential "
                                     "which handles exactly one separation!".format(self.__class__.__name__))
        if charge is not None and potential.number_charge_arguments != 2:
            raise ConfigurationError("The event handler {0} was initialized with a charge which is not None,"
                                     " but its potential {1} expects not exactly 2 charges."
                                     .format(self.__class__.__name__, potential.__class__.__name__))
        self._potential = potential
        self._charge = charge
        self._target_index = None

    def _potential_change(self, target_unit) -> float:
        """The potential change of the pair with ``target_unit`` (two_leaf_unit_event_handler.py:95-98)."""
        return random.expovariate(setting.beta)

    def send_event_time(self, in_state: Sequence[Node]) -> Time:
        """The candidate event time: the earliest pair event of the active leaf unit in the in-state (the active
        unit's branch and the branches of its targets).  Every unit of the in-state is time-sliced to it."""
        self._store_in_state(in_state)
        self._construct_leaf_cnodes()
        self._extract_active_leaf_unit()
        active = self._active_leaf_unit
        targets = [i for i in range(len(self._leaf_units)) if i != self._active_leaf_unit_index]
        separations = [setting.periodic_boundaries.separation_vector(active.position, self._leaf_units[i].position)
                       for i in targets]
        if self._charge is None:
            charges = [(1.0, 1.0)] * len(targets)
        else:
            charges = [(active.charge[self._charge], self._leaf_units[i].charge[self._charge]) for i in targets]
        if self._potential.potential_change_required:
            changes = [self._potential_change(self._leaf_units[i]) for i in targets]
        else:
            changes = [0.0] * len(targets)
        index, displacement = earliest(self._potential, active.velocity, separations, charges, changes)
        self._target_index = targets[index] if index >= 0 else None
        self._event_time = active.time_stamp + displacement
        self._time_slice_all_units_in_state()
        return self._event_time

    def send_out_state(self) -> Sequence[Node]:
        """The out-state: the velocity of the active leaf unit moves to the target of the earliest pair event."""
        self._exchange_velocity(self._leaf_cnodes[self._active_leaf_unit_index],
                                self._leaf_cnodes[self._target_index])
        return self._state
