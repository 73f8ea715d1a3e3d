"""GPU drop-in for ``LennardJonesPotential`` (``potential/lennard_jones_potential.py:43-135`` with the Mexican-hat
inversion of ``potential/abstracts.py:336-530``)."""
from typing import Sequence

from jellyfysh_gb300 import potentials
from jellyfysh_gb300.plugin.potential._common import GpuPotential


class GpuLennardJonesPotential(GpuPotential):
    """U(r) = k ((s / r)^12 - (s / r)^6) with k the prefactor and s the characteristic length.  The separation
    argument is not mutated (the reference mutates it while it slides; its callers pass a fresh list)."""

    def __init__(self, prefactor: float = 1.0, characteristic_length: float = 1.0):
        if prefactor == 0.0:
            raise ValueError("Give a prefactor unequal 0.0 as the prefactor for the potential {0}."
                             .format(self.__class__.__name__))
        self._prefactor = prefactor
        self._characteristic_length = characteristic_length

    def displacement(self, velocity: Sequence[float], separation: Sequence[float], potential_change: float) -> float:
        return self._one(potentials.lennard_jones_displacement(self._prefactor, self._characteristic_length, velocity,
                                                               separation, potential_change))

    def displacements(self, velocity, separations, charges, potential_changes):
        return potentials.lennard_jones_displacement(self._prefactor, self._characteristic_length, velocity,
                                                     separations, potential_changes)

    def derivative(self, velocity: Sequence[float], separation: Sequence[float]) -> float:
        return self._one(potentials.lennard_jones_derivative(self._prefactor, self._characteristic_length, velocity,
                                                             separation))
