"""GPU drop-in for ``InversePowerPotential`` (``potential/inverse_power_potential.py:43-179``)."""
from typing import Sequence

from jellyfysh_gb300 import potentials
from jellyfysh_gb300.plugin.potential._common import GpuPotential


class GpuInversePowerPotential(GpuPotential):
    """U = k c1 c2 / r^p for the power p and the prefactor k."""

    charges = 2

    def __init__(self, power: float, prefactor: float) -> None:
        if prefactor == 0.0:
            raise ValueError("Give a prefactor unequal 0.0 as the prefactor for the potential {0}."
                             .format(self.__class__.__name__))
        if not power > 0.0:
            raise ValueError("the power of the potential {0} must be positive".format(self.__class__.__name__))
        self._power = power
        self._prefactor = prefactor

    def displacement(self, velocity: Sequence[float], separation: Sequence[float], charge_one: float,
                     charge_two: float, potential_change: float) -> float:
        return self._one(potentials.inverse_power_displacement(self._power, self._prefactor, velocity, separation,
                                                               [charge_one, charge_two], potential_change))

    def displacements(self, velocity, separations, charges, potential_changes):
        return potentials.inverse_power_displacement(self._power, self._prefactor, velocity, separations, charges,
                                                     potential_changes)

    def derivative(self, velocity: Sequence[float], separation: Sequence[float], charge_one: float,
                   charge_two: float) -> float:
        return self._one(potentials.inverse_power_derivative(self._power, self._prefactor, velocity, separation,
                                                             [charge_one, charge_two]))
