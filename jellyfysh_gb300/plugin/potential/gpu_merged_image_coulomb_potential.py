"""GPU drop-in for ``MergedImageCoulombPotential``
(``potential/merged_image_coulomb_potential/merged_image_coulomb_potential.py:61-154``, the Ewald sum of
``merged_image_coulomb_potential.c:77-274``)."""
from typing import Sequence

from jellyfysh_gb300 import potentials
from jellyfysh_gb300.plugin.potential._common import GpuPotential, system_length


class GpuMergedImageCoulombPotential(GpuPotential):
    """Coulomb interaction of a charge with all periodic images of another (Ewald summation with the splitting
    parameter alpha over the Fourier and position cutoffs), in the periodic cube of the setting.  Like the
    reference's, it has a derivative only."""

    charges = 2

    def __init__(self, alpha: float = 3.45, fourier_cutoff: int = 6, position_cutoff: int = 2,
                 prefactor: float = 1.0) -> None:
        if prefactor == 0.0:
            raise ValueError("Give a prefactor unequal 0.0 as the prefactor for the potential {0}."
                             .format(self.__class__.__name__))
        self._alpha = alpha
        self._fourier_cutoff = fourier_cutoff
        self._position_cutoff = position_cutoff
        self._prefactor = prefactor
        self._system_length = None

    def derivative(self, velocity: Sequence[float], separation: Sequence[float], charge_one: float,
                   charge_two: float) -> float:
        if self._system_length is None:
            self._system_length = system_length()
        return self._one(potentials.merged_image_coulomb_derivative(
            self._alpha, self._fourier_cutoff, self._position_cutoff, self._prefactor, self._system_length,
            velocity, separation, [charge_one, charge_two]))
