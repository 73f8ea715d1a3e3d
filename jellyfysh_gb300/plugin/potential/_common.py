"""Properties the reference's event handlers read from a potential (``potential/potential.py:76-151, 262-301``), and
the batched earliest pair event of a whole neighbourhood."""
import numpy as np

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

    def displacements(self, velocity, separations, charges, potential_changes):
        """The displacements of one active unit against n targets in one launch: ``velocity`` [3], ``separations``
        [n][3], ``charges`` [n][2] (ignored by uncharged potentials), ``potential_changes`` [n] (ignored when the
        potential wants none).  Returns host arrays (time displacements [n], JFGPU_STATUS_* [n])."""
        raise NotImplementedError("the potential {0} has no batched displacement".format(self.__class__.__name__))


def system_length(explicit=None) -> float:
    """The box side: an explicit value, else the reference's hypercubic setting
    (``setting/hypercubic_setting.py:39-67``)."""
    if explicit is not None:
        return float(explicit)
    from jellyfysh.setting import hypercubic_setting as setting
    if not setting.initialized() or setting.dimension != 3:
        raise ValueError("the potential needs a three-dimensional hypercubic setting")
    return float(setting.system_length)


def earliest(potential, velocity, separations, charges, potential_changes):
    """The earliest pair event of one active unit against n targets: one batched launch of the potential's
    displacements, then the smallest (the first of equal ones, in the targets' order).  Returns (index, displacement),
    index -1 and displacement inf when no target has an event; raises the reference's exception of the first target
    whose solve raised one."""
    if len(separations) == 0:
        return -1, float("inf")
    out, status = potential.displacements(velocity, separations, charges, potential_changes)
    failed = np.nonzero(status)[0]
    if failed.size:
        potentials.raise_status(int(status[failed[0]]))
    index = int(np.argmin(out))
    if np.isinf(out[index]):
        return -1, float("inf")
    return index, float(out[index])
