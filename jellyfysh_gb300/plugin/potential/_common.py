"""Properties the reference's event handlers read from a potential (``potential/potential.py:76-151, 262-301``)."""
from jellyfysh_gb300 import potentials


class GpuPotential:
    """Declares the argument counts that the reference would inspect from the method signatures: the number of
    separation and charge arguments of ``derivative`` and whether ``displacement`` wants a potential change."""

    separations = 1
    charges = 0
    wants_potential_change = True

    @property
    def number_separation_arguments(self) -> int:
        return self.separations

    @property
    def number_charge_arguments(self) -> int:
        return self.charges

    @property
    def potential_change_required(self) -> bool:
        return self.wants_potential_change

    @staticmethod
    def _one(result) -> float:
        return potentials.single(result)


def system_length(explicit=None) -> float:
    """The box side: an explicit value, else the reference's hypercubic setting
    (``setting/hypercubic_setting.py:39-67``)."""
    if explicit is not None:
        return float(explicit)
    from jellyfysh.setting import hypercubic_setting as setting
    if not setting.initialized() or setting.dimension != 3:
        raise ValueError("the potential needs a three-dimensional hypercubic setting")
    return float(setting.system_length)
