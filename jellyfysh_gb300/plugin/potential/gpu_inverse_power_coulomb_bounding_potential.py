"""GPU drop-in for ``InversePowerCoulombBoundingPotential``
(``potential/inverse_power_coulomb_bounding_potential/inverse_power_coulomb_bounding_potential.py:58-140``, the
arithmetic of ``inverse_power_coulomb_bounding_potential.c:85-139``)."""
from typing import Sequence

from jellyfysh_gb300 import potentials
from jellyfysh_gb300.plugin.potential._common import GpuPotential, system_length


class GpuInversePowerCoulombBoundingPotential(GpuPotential):
    """Nearest-image 1/r bound of the merged-image Coulomb potential in the periodic cube of the setting."""

    charges = 2

    def __init__(self, prefactor: float = 1.5837) -> None:
        self._prefactor = prefactor
        self._system_length = None

    def _length(self) -> float:
        if self._system_length is None:
            self._system_length = system_length()
        return self._system_length

    def displacement(self, velocity: Sequence[float], separation: Sequence[float], charge_one: float,
                     charge_two: float, potential_change: float) -> float:
        return self._one(potentials.coulomb_bound_displacement(self._prefactor, self._length(), velocity,
                                                               separation, [charge_one, charge_two],
                                                               potential_change))

    def displacements(self, velocity, separations, charges, potential_changes):
        return potentials.coulomb_bound_displacement(self._prefactor, self._length(), velocity, separations, charges,
                                                     potential_changes)

    def derivative(self, velocity: Sequence[float], separation: Sequence[float], charge_one: float,
                   charge_two: float) -> float:
        return self._one(potentials.coulomb_bound_derivative(self._prefactor, velocity, separation,
                                                             [charge_one, charge_two]))
