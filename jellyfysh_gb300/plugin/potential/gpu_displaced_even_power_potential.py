"""GPU drop-in for ``DisplacedEvenPowerPotential`` (``potential/displaced_even_power_potential.py:44-142``)."""
from typing import Sequence

from jellyfysh_gb300 import potentials
from jellyfysh_gb300.plugin.potential._common import GpuPotential


class GpuDisplacedEvenPowerPotential(GpuPotential):
    """U = k (r - r0)^n for an even power n (harmonic bonds for n = 2)."""

    def __init__(self, equilibrium_separation: float, power: int, prefactor: float = 1.0) -> None:
        if power <= 0 or power % 2:
            raise ValueError("the power of the potential {0} must be even and positive"
                             .format(self.__class__.__name__))
        if prefactor == 0.0:
            raise ValueError("Give a prefactor unequal 0.0 as the prefactor for the potential {0}."
                             .format(self.__class__.__name__))
        self._equilibrium_separation = equilibrium_separation
        self._power = power
        self._prefactor = prefactor

    def displacement(self, velocity: Sequence[float], separation: Sequence[float], potential_change: float) -> float:
        return self._one(potentials.displaced_even_power_displacement(
            self._equilibrium_separation, self._power, self._prefactor, velocity, separation, potential_change))

    def displacements(self, velocity, separations, charges, potential_changes):
        return potentials.displaced_even_power_displacement(self._equilibrium_separation, self._power,
                                                            self._prefactor, velocity, separations, potential_changes)

    def derivative(self, velocity: Sequence[float], separation: Sequence[float]) -> float:
        return self._one(potentials.displaced_even_power_derivative(
            self._equilibrium_separation, self._power, self._prefactor, velocity, separation))
