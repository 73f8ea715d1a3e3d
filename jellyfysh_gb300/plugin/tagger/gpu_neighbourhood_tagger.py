"""Tagger of whole neighbourhoods for the GPU neighbourhood event handler.

The reference's ExcludedCellsTagger (``activator/tagger/excluded_cells_tagger.py:107-132``) and SurplusCellsTagger
(``activator/tagger/surplus_cells_tagger.py:107-131``) yield one pairwise in-state per (active unit, target) of the
nearby cells and of the surplus.  ``GpuNeighbourhoodTagger`` yields, per active unit of the cell-occupancy system, one
in-state with the active unit and all of those targets together (nearby-cell occupants in the order of
``nearby_cells``, then the surplus units), the way ``cell_bounding_potential_tagger.py:150-155`` yields in-states of
variable length, so that one event handler solves the whole neighbourhood at once.
"""
import logging
from typing import Iterable, Sequence, Tuple

from jellyfysh.activator.internal_state import CellOccupancy, InternalState
from jellyfysh.activator.tagger.abstracts import TaggerWithInternalState
from jellyfysh.base.exceptions import ConfigurationError
from jellyfysh.base.logging import log_init_arguments
from jellyfysh.base.node import Node
from jellyfysh.event_handler import EventHandler


class GpuNeighbourhoodTagger(TaggerWithInternalState):
    """One in-state per active unit of the cell-occupancy system: the active unit, every occupant of its nearby
    cells and every surplus unit.  Works with a cell-occupancy internal state only."""

    def __init__(self, create: Sequence[str], trash: Sequence[str], event_handler: EventHandler,
                 internal_state_label: str, number_event_handlers: int = 1, tag: str = None) -> None:
        log_init_arguments(logging.getLogger(__name__).debug, self.__class__.__name__,
                           event_handler=event_handler.__class__.__name__, number_event_handlers=number_event_handlers,
                           internal_state_label=internal_state_label, create=create, trash=trash, tag=tag)
        super().__init__(create, trash, event_handler, internal_state_label=internal_state_label,
                         number_event_handlers=number_event_handlers, tag=tag)

    def initialize_with_internal_states(self, internal_states: Sequence[InternalState]) -> None:
        """Check that the internal state is a cell-occupancy system."""
        super().initialize_with_internal_states(internal_states)
        if not isinstance(self._internal_state, CellOccupancy):
            raise ConfigurationError("The tagger {0} can only be used with an instance of the CellOccupancy class as "
                                     "the internal state.".format(self.__class__.__name__))

    def yield_identifiers_send_event_time(self, extracted_active_global_state: Sequence[Node]) -> Iterable[Tuple]:
        """The in-state identifiers: per active cell, the active identifier followed by all nearby occupants and
        surplus identifiers."""
        for active_cell, active_identifier in self._internal_state.yield_active_cells():
            nearby = tuple(occupant for nearby_cell in self._internal_state.cells.nearby_cells(active_cell)
                           for occupant in self._internal_state[nearby_cell])
            surplus = tuple(self._internal_state.yield_surplus())
            yield (active_identifier,) + nearby + surplus
