"""GPU drop-in for ``HardSpherePotential`` (``potential/hard_sphere_potential.py:44-125``)."""
from typing import Sequence

from jellyfysh_gb300 import potentials
from jellyfysh_gb300.plugin.potential._common import GpuPotential


class GpuHardSpherePotential(GpuPotential):
    """Hard spheres of the given radius: the collision time of the active sphere moving along the velocity."""

    wants_potential_change = False

    def __init__(self, radius: float) -> None:
        if not radius > 0.0:
            raise ValueError("the radius of the hard spheres must be positive")
        self._radius = radius

    def displacement(self, velocity: Sequence[float], separation: Sequence[float]) -> float:
        return self._one(potentials.hard_sphere_displacement(self._radius, velocity, separation))

    def displacements(self, velocity, separations, charges, potential_changes):
        return potentials.hard_sphere_displacement(self._radius, velocity, separations)

    def derivative(self, velocity: Sequence[float], separation: Sequence[float]) -> float:
        raise NotImplementedError("The derivative method of the class {0} should not be used."
                                  .format(self.__class__.__name__))
