"""Events between two composite objects on the GPU: dipoles and water molecules whose point charges interact by the
merged-image Coulomb potential, bounded pair by pair by the inverse-power Coulomb bound and summed over the target
object (``TwoCompositeObjectSummedBoundingPotentialEventHandler``,
``event_handler/two_composite_object_summed_bounding_potential_event_handler.py:119-202``).

``event_time`` is the handler's ``send_event_time`` and ``out_state`` its ``send_out_state`` (thinning, the
derivative table of ``_fill_lifting`` and the lifting scheme) for n events in one launch each, through
``jfgpu_composite_event_time`` / ``jfgpu_composite_out_state`` (``include/jfgpu.h``).
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib

LIFTING = {"inside_first": _lib.LIFTING_INSIDE_FIRST, "outside_first": _lib.LIFTING_OUTSIDE_FIRST,
           "ratio": _lib.LIFTING_RATIO}


@dataclass
class CompositeModel:
    """Two composite objects of ``units`` charges each; defaults are the reference's constructor defaults
    (``MergedImageCoulombPotential``: alpha 3.45, Fourier cutoff 6, position cutoff 2, prefactor 1;
    ``InversePowerCoulombBoundingPotential``: prefactor 1.5837)."""

    units: int
    system_length: float
    lifting: str = "inside_first"
    alpha: float = 3.45
    fourier_cutoff: int = 6
    position_cutoff: int = 2
    coulomb_prefactor: float = 1.0
    bound_prefactor: float = 1.5837

    def desc(self) -> "_lib.CompositeDesc":
        return _lib.CompositeDesc(units=int(self.units), lifting=LIFTING[self.lifting],
                                  fourier_cutoff=int(self.fourier_cutoff), position_cutoff=int(self.position_cutoff),
                                  alpha=float(self.alpha), coulomb_prefactor=float(self.coulomb_prefactor),
                                  bound_prefactor=float(self.bound_prefactor),
                                  system_length=float(self.system_length))


def _device():
    import torch
    return torch, torch.device("cuda", torch.cuda.current_device())


def _on_device(torch, device, values, dtype, shape):
    if isinstance(values, torch.Tensor) and values.is_cuda:
        tensor = values.to(dtype).contiguous()
    else:
        tensor = torch.as_tensor(np.ascontiguousarray(np.asarray(values)), dtype=dtype).to(device)
    return tensor.reshape(shape)


def event_time(model: CompositeModel, velocity, active_position, active_charge, target_positions, target_charges,
               potential_changes):
    """Candidate displacement of n events: (displacement [n], status [n]) as host arrays.  velocity and
    active_position [n][3], active_charge [n], target_positions [n][units][3], target_charges and
    potential_changes [n][units]."""
    torch, device = _device()
    lib = _lib.load()
    k = model.units
    v = _on_device(torch, device, velocity, torch.float64, (-1, 3))
    n = v.shape[0]
    arrays = [v, _on_device(torch, device, active_position, torch.float64, (n, 3)),
              _on_device(torch, device, active_charge, torch.float64, (n,)),
              _on_device(torch, device, target_positions, torch.float64, (n, k, 3)),
              _on_device(torch, device, target_charges, torch.float64, (n, k)),
              _on_device(torch, device, potential_changes, torch.float64, (n, k))]
    out = torch.empty(max(n, 1), dtype=torch.float64, device=device)
    status = torch.empty(max(n, 1), dtype=torch.int32, device=device)
    desc = model.desc()
    stream = torch.cuda.current_stream(device).cuda_stream
    _lib.check(lib.jfgpu_composite_event_time(ctypes.byref(desc), *[a.data_ptr() for a in arrays], n,
                                              out.data_ptr(), status.data_ptr(), stream),
               "jfgpu_composite_event_time")
    return out[:n].cpu().numpy(), status[:n].cpu().numpy()


def out_state(model: CompositeModel, velocity, local_positions, local_charges, active_index, target_positions,
              target_charges, local_first, draws, unit_draws: bool = False):
    """Out-state of n events: (new_active [n], rates [n][2], status [n]) as host arrays.  new_active is -1 for a
    thinned event, i for local unit i and units + j for target unit j; rates hold the summed bounding event rate and
    the event rate.  draws [n][3]: thinning, lifting insert, ratio draw (values, or unit draws with
    ``unit_draws``)."""
    torch, device = _device()
    lib = _lib.load()
    k = model.units
    v = _on_device(torch, device, velocity, torch.float64, (-1, 3))
    n = v.shape[0]
    arrays = [v, _on_device(torch, device, local_positions, torch.float64, (n, k, 3)),
              _on_device(torch, device, local_charges, torch.float64, (n, k)),
              _on_device(torch, device, active_index, torch.int32, (n,)),
              _on_device(torch, device, target_positions, torch.float64, (n, k, 3)),
              _on_device(torch, device, target_charges, torch.float64, (n, k)),
              _on_device(torch, device, local_first, torch.int32, (n,)),
              _on_device(torch, device, draws, torch.float64, (n, 3))]
    new_active = torch.empty(max(n, 1), dtype=torch.int32, device=device)
    rates = torch.empty((max(n, 1), 2), dtype=torch.float64, device=device)
    status = torch.empty(max(n, 1), dtype=torch.int32, device=device)
    desc = model.desc()
    stream = torch.cuda.current_stream(device).cuda_stream
    _lib.check(lib.jfgpu_composite_out_state(ctypes.byref(desc), _lib.DRAW_UNIT if unit_draws else _lib.DRAW_VALUE,
                                             *[a.data_ptr() for a in arrays], n, new_active.data_ptr(),
                                             rates.data_ptr(), status.data_ptr(), stream),
               "jfgpu_composite_out_state")
    return new_active[:n].cpu().numpy(), rates[:n].cpu().numpy(), status[:n].cpu().numpy()
