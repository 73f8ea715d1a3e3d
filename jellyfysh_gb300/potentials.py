"""Batched pair potentials on the GPU: host arrays in, host arrays out, through the C ABI.

Each function evaluates the reference's ``displacement`` or ``derivative`` (``potential/potential.py:153-253``) of
one potential for n (velocity, separation[, charges][, potential change]) rows in one launch.  Per-row status codes
come back as the exceptions the reference raises (``raise_status``); ``inf`` means "no event", as in the reference.
The arithmetic is the reference's, in FP64 on the device (see the C ABI in ``include/jfgpu.h``).
"""
from typing import Optional

import numpy as np

from . import _lib

_STATUS_EXCEPTIONS = {
    _lib.STATUS_VALUE_ERROR: (ValueError, "math domain error"),        # math.sqrt of a negative number
    _lib.STATUS_ASSERTION: (AssertionError, "assertion of the reference failed"),
    _lib.STATUS_ZERO_DIVISION: (ZeroDivisionError, "float division by zero"),
    _lib.STATUS_COMPLEX: (TypeError, "negative number raised to a fractional power (complex result)"),
}


def raise_status(status: int) -> None:
    """Raise the reference's exception for a JFGPU_STATUS_* code (nothing for JFGPU_STATUS_OK)."""
    if status:
        kind, message = _STATUS_EXCEPTIONS.get(int(status), (RuntimeError, "status %d" % int(status)))
        raise kind(message)


class _Device:
    """Device buffers of one batched call (PyTorch tensors as plain device memory)."""

    def __init__(self):
        import torch
        self.torch = torch
        self.lib = _lib.load()
        self.device = torch.device("cuda", torch.cuda.current_device())

    def array(self, values, columns: Optional[int] = None):
        torch = self.torch
        a = np.ascontiguousarray(np.asarray(values, dtype=np.float64))
        if columns is not None:
            a = a.reshape(-1, columns)
        return torch.from_numpy(a).to(self.device)

    def call(self, function, scalars, arrays, n):
        torch = self.torch
        out = torch.empty(n, dtype=torch.float64, device=self.device)
        status = torch.empty(n, dtype=torch.int32, device=self.device)
        stream = torch.cuda.current_stream(self.device).cuda_stream
        pointers = [a.data_ptr() if a is not None else None for a in arrays]
        _lib.check(getattr(self.lib, function)(*scalars, *pointers, n, out.data_ptr(), status.data_ptr(), stream),
                   function)
        return out.cpu().numpy(), status.cpu().numpy()


_device: Optional[_Device] = None


def _dev() -> _Device:
    global _device
    if _device is None:
        _device = _Device()
    return _device


def _rows(velocities, separations):
    v = np.asarray(velocities, dtype=np.float64).reshape(-1, 3)
    s = np.asarray(separations, dtype=np.float64).reshape(-1, 3)
    n = max(len(v), len(s))
    if len(v) == 1 and n > 1:
        v = np.repeat(v, n, axis=0)
    return v, s, n


def _charges(charges, n):
    c = np.asarray(charges, dtype=np.float64).reshape(-1, 2)
    return np.repeat(c, n, axis=0) if len(c) == 1 and n > 1 else c


def _column(values, n):
    c = np.asarray(values, dtype=np.float64).reshape(-1)
    return np.repeat(c, n) if len(c) == 1 and n > 1 else c


def hard_sphere_displacement(radius, velocities, separations):
    """HardSpherePotential.displacement (hard_sphere_potential.py:65-99): (out [n], status [n])."""
    d = _dev()
    v, s, n = _rows(velocities, separations)
    return d.call("jfgpu_hard_sphere_displacement", (float(radius),), (d.array(v), d.array(s)), n)


def inverse_power_displacement(power, prefactor, velocities, separations, charges, potential_changes):
    """InversePowerPotential.displacement (inverse_power_potential.py:96-179)."""
    d = _dev()
    v, s, n = _rows(velocities, separations)
    return d.call("jfgpu_inverse_power_displacement", (float(power), float(prefactor)),
                  (d.array(v), d.array(s), d.array(_charges(charges, n)), d.array(_column(potential_changes, n))), n)


def inverse_power_derivative(power, prefactor, velocities, separations, charges):
    """InversePowerPotential.derivative (inverse_power_potential.py:71-94)."""
    d = _dev()
    v, s, n = _rows(velocities, separations)
    return d.call("jfgpu_inverse_power_derivative", (float(power), float(prefactor)),
                  (d.array(v), d.array(s), d.array(_charges(charges, n))), n)


def lennard_jones_displacement(prefactor, characteristic_length, velocities, separations, potential_changes):
    """LennardJonesPotential.displacement (abstracts.py:336-530 with lennard_jones_potential.py:100-135)."""
    d = _dev()
    v, s, n = _rows(velocities, separations)
    return d.call("jfgpu_lennard_jones_displacement", (float(prefactor), float(characteristic_length)),
                  (d.array(v), d.array(s), d.array(_column(potential_changes, n))), n)


def lennard_jones_derivative(prefactor, characteristic_length, velocities, separations):
    """LennardJonesPotential.derivative (lennard_jones_potential.py:63-81)."""
    d = _dev()
    v, s, n = _rows(velocities, separations)
    return d.call("jfgpu_lennard_jones_derivative", (float(prefactor), float(characteristic_length)),
                  (d.array(v), d.array(s)), n)


def displaced_even_power_displacement(equilibrium_separation, power, prefactor, velocities, separations,
                                      potential_changes):
    """DisplacedEvenPowerPotential.displacement (displaced_even_power_potential.py:73-142)."""
    d = _dev()
    v, s, n = _rows(velocities, separations)
    return d.call("jfgpu_displaced_even_power_displacement",
                  (float(equilibrium_separation), int(power), float(prefactor)),
                  (d.array(v), d.array(s), d.array(_column(potential_changes, n))), n)


def displaced_even_power_derivative(equilibrium_separation, power, prefactor, velocities, separations):
    """DisplacedEvenPowerPotential.derivative (displaced_even_power_potential.py:73-90)."""
    d = _dev()
    v, s, n = _rows(velocities, separations)
    return d.call("jfgpu_displaced_even_power_derivative",
                  (float(equilibrium_separation), int(power), float(prefactor)), (d.array(v), d.array(s)), n)


def coulomb_bound_displacement(prefactor, system_length, velocities, separations, charges, potential_changes):
    """InversePowerCoulombBoundingPotential.displacement (inverse_power_coulomb_bounding_potential.py:111-140,
    inverse_power_coulomb_bounding_potential.c:85-139)."""
    d = _dev()
    v, s, n = _rows(velocities, separations)
    return d.call("jfgpu_coulomb_bound_displacement", (float(prefactor), float(system_length)),
                  (d.array(v), d.array(s), d.array(_charges(charges, n)), d.array(_column(potential_changes, n))), n)


def coulomb_bound_derivative(prefactor, velocities, separations, charges):
    """InversePowerCoulombBoundingPotential.derivative (inverse_power_coulomb_bounding_potential.py:84-109)."""
    d = _dev()
    v, s, n = _rows(velocities, separations)
    return d.call("jfgpu_coulomb_bound_derivative", (float(prefactor),),
                  (d.array(v), d.array(s), d.array(_charges(charges, n))), n)


def merged_image_coulomb_derivative(alpha, fourier_cutoff, position_cutoff, prefactor, system_length, velocities,
                                    separations, charges):
    """MergedImageCoulombPotential.derivative (merged_image_coulomb_potential.py:128-154,
    merged_image_coulomb_potential.c:205-274)."""
    d = _dev()
    v, s, n = _rows(velocities, separations)
    return d.call("jfgpu_merged_image_coulomb_derivative",
                  (float(alpha), int(fourier_cutoff), int(position_cutoff), float(prefactor), float(system_length)),
                  (d.array(v), d.array(s), d.array(_charges(charges, n))), n)


def single(result) -> float:
    """The value of a one-row call, or the reference's exception for its status."""
    out, status = result
    raise_status(status[0])
    return float(out[0])

