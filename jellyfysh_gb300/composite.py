"""Events between two composite objects on the GPU: dipoles and water molecules whose point charges interact by the
merged-image Coulomb potential, bounded pair by pair by the inverse-power Coulomb bound and summed over the target
object (``TwoCompositeObjectSummedBoundingPotentialEventHandler``,
``event_handler/two_composite_object_summed_bounding_potential_event_handler.py:119-202``).

``event_time`` is the handler's ``send_event_time`` and ``out_state`` its ``send_out_state`` (thinning, the
derivative table of ``_fill_lifting`` and the lifting scheme) for n events in one launch each, through
``jfgpu_composite_event_time`` / ``jfgpu_composite_out_state`` (``include/jfgpu.h``).

The far field between composite objects: ``cell_bound_time`` is the event time of the molecular cell-bounding
handler (``TwoCompositeObjectCellBoundingPotentialEventHandler``,
``event_handler/two_composite_object_cell_bounding_potential_event_handler.py:153-265``), ``cell_veto_time`` that of
the molecular cell veto for sampled relative cells (``CompositeObjectCellVetoEventHandler``,
``event_handler/composite_object_cell_veto_event_handler.py:110-162``), and ``bounded_out_state`` the out-state of
both: the summed merged-image derivative thinned against the given bounding event rate, then the lifting.
``WalkerTable`` / ``walker_sample`` build the cell veto's alias table and sample its relative cells.
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


def bounded_out_state(model: CompositeModel, velocity, local_positions, local_charges, active_index,
                      target_positions, target_charges, local_first, bounding_rates, draws, unit_draws: bool = False):
    """Out-state of n events of the molecular cell-bounding or cell-veto handler: as ``out_state``, with the thinning
    drawn against bounding_rates [n] (the cell-bounding rate times the speed, or the cell veto's rate)."""
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
              _on_device(torch, device, bounding_rates, torch.float64, (n,)),
              _on_device(torch, device, draws, torch.float64, (n, 3))]
    new_active = torch.empty(max(n, 1), dtype=torch.int32, device=device)
    rates = torch.empty((max(n, 1), 2), dtype=torch.float64, device=device)
    status = torch.empty(max(n, 1), dtype=torch.int32, device=device)
    desc = model.desc()
    stream = torch.cuda.current_stream(device).cuda_stream
    _lib.check(lib.jfgpu_composite_bounded_out_state(
        ctypes.byref(desc), _lib.DRAW_UNIT if unit_draws else _lib.DRAW_VALUE, *[a.data_ptr() for a in arrays], n,
        new_active.data_ptr(), rates.data_ptr(), status.data_ptr(), stream), "jfgpu_composite_bounded_out_state")
    return new_active[:n].cpu().numpy(), rates[:n].cpu().numpy(), status[:n].cpu().numpy()


class CellBounds:
    """The estimator's derivative bounds of the far cells, on the device: upper and lower [cells][3] by relative cell
    (the cuboid cell index, x fastest) and direction, NaN for the nearby cells; for the cell veto also the Walker
    tables' total rates by direction."""

    def __init__(self, upper, lower, walker_upper=None, walker_lower=None):
        torch, device = _device()
        upper = np.asarray(upper, dtype=np.float64).reshape(-1, 3)
        lower = np.asarray(lower, dtype=np.float64).reshape(-1, 3)
        if upper.shape != lower.shape:
            raise ValueError("upper and lower bounds differ in shape")
        self.cells = upper.shape[0]
        self.upper = torch.from_numpy(np.ascontiguousarray(upper)).to(device)
        self.lower = torch.from_numpy(np.ascontiguousarray(lower)).to(device)
        self.walker_upper = self.walker_lower = None
        if walker_upper is not None:
            self.walker_upper = torch.as_tensor(np.asarray(walker_upper, dtype=np.float64).reshape(3)).to(device)
            self.walker_lower = torch.as_tensor(np.asarray(walker_lower, dtype=np.float64).reshape(3)).to(device)


def cell_bound_time(bounds: CellBounds, relative_cell, velocity, active_charge, target_charges, dipole_charge,
                    potential_change):
    """Event time of n molecular cell-bounding events: (rate [n], time displacement [n], status [n]) as host
    arrays.  relative_cell [n], velocity [n][3], active_charge [n], target_charges [n][units], potential_change
    [n]."""
    torch, device = _device()
    lib = _lib.load()
    v = _on_device(torch, device, velocity, torch.float64, (-1, 3))
    n = v.shape[0]
    charges = _on_device(torch, device, target_charges, torch.float64, (n, -1)) if n else \
        torch.zeros((0, 1), dtype=torch.float64, device=device)
    units = charges.shape[1]
    arrays = [_on_device(torch, device, relative_cell, torch.int32, (n,)), v,
              _on_device(torch, device, active_charge, torch.float64, (n,)), charges]
    du = _on_device(torch, device, potential_change, torch.float64, (n,))
    rate = torch.empty(max(n, 1), dtype=torch.float64, device=device)
    time = torch.empty(max(n, 1), dtype=torch.float64, device=device)
    status = torch.empty(max(n, 1), dtype=torch.int32, device=device)
    stream = torch.cuda.current_stream(device).cuda_stream
    _lib.check(lib.jfgpu_composite_cell_bound_time(
        bounds.upper.data_ptr(), bounds.lower.data_ptr(), bounds.cells, *[a.data_ptr() for a in arrays], units,
        float(dipole_charge), du.data_ptr(), n, rate.data_ptr(), time.data_ptr(), status.data_ptr(), stream),
        "jfgpu_composite_cell_bound_time")
    return rate[:n].cpu().numpy(), time[:n].cpu().numpy(), status[:n].cpu().numpy()


def cell_veto_time(bounds: CellBounds, relative_cell, velocity, active_charge, potential_change):
    """Event time of n molecular cell-veto events for sampled relative cells: (rate [n], time displacement [n],
    status [n]) as host arrays."""
    if bounds.walker_upper is None:
        raise ValueError("the cell veto needs the Walker tables' total rates")
    torch, device = _device()
    lib = _lib.load()
    v = _on_device(torch, device, velocity, torch.float64, (-1, 3))
    n = v.shape[0]
    arrays = [_on_device(torch, device, relative_cell, torch.int32, (n,)), v,
              _on_device(torch, device, active_charge, torch.float64, (n,)),
              _on_device(torch, device, potential_change, torch.float64, (n,))]
    rate = torch.empty(max(n, 1), dtype=torch.float64, device=device)
    time = torch.empty(max(n, 1), dtype=torch.float64, device=device)
    status = torch.empty(max(n, 1), dtype=torch.int32, device=device)
    stream = torch.cuda.current_stream(device).cuda_stream
    _lib.check(lib.jfgpu_composite_cell_veto_time(
        bounds.upper.data_ptr(), bounds.lower.data_ptr(), bounds.cells, bounds.walker_upper.data_ptr(),
        bounds.walker_lower.data_ptr(), *[a.data_ptr() for a in arrays], n, rate.data_ptr(), time.data_ptr(),
        status.data_ptr(), stream), "jfgpu_composite_cell_veto_time")
    return rate[:n].cpu().numpy(), time[:n].cpu().numpy(), status[:n].cpu().numpy()


class WalkerTable:
    """Walker's alias table (``event_handler/walker.py:53-103``) built on the host in the reference's order and held
    on the device: ``items`` the relative cells and ``rates`` their rates, in the order the handler lists them."""

    def __init__(self, items, rates):
        torch, device = _device()
        lib = _lib.load()
        items = np.ascontiguousarray(np.asarray(items, dtype=np.int32))
        rates = np.ascontiguousarray(np.asarray(rates, dtype=np.float64))
        n = len(items)
        if len(rates) != n:
            raise ValueError("one rate per item is required")
        first_item = np.zeros(max(n, 1), dtype=np.int32)
        second_item = np.zeros(max(n, 1), dtype=np.int32)
        first_rate = np.zeros(max(n, 1), dtype=np.float64)
        total, mean = ctypes.c_double(0.0), ctypes.c_double(0.0)
        _lib.check(lib.jfgpu_walker_table(items.ctypes.data, rates.ctypes.data, n, first_item.ctypes.data,
                                          first_rate.ctypes.data, second_item.ctypes.data, ctypes.byref(total),
                                          ctypes.byref(mean)), "jfgpu_walker_table")
        self.size = n
        self.total_rate, self.mean_rate = total.value, mean.value
        self.first_item_host, self.first_rate_host, self.second_item_host = first_item, first_rate, second_item
        self.first_item = torch.from_numpy(first_item).to(device)
        self.first_rate = torch.from_numpy(first_rate).to(device)
        self.second_item = torch.from_numpy(second_item).to(device)


def walker_sample(table: WalkerTable, choices, draws, unit_draws: bool = False):
    """Walker.sample_cell (``walker.py:105-122``) for n draws: (items [n], status [n]) as host arrays.  choices [n]
    are table indices (what random.choice picked), draws [n] the random.uniform(0.0, mean rate) values, or unit draws
    with ``unit_draws``."""
    torch, device = _device()
    lib = _lib.load()
    k = _on_device(torch, device, choices, torch.int64, (-1,))
    n = k.shape[0]
    u = _on_device(torch, device, draws, torch.float64, (n,))
    items = torch.empty(max(n, 1), dtype=torch.int32, device=device)
    status = torch.empty(max(n, 1), dtype=torch.int32, device=device)
    stream = torch.cuda.current_stream(device).cuda_stream
    _lib.check(lib.jfgpu_walker_sample(table.first_item.data_ptr(), table.first_rate.data_ptr(),
                                       table.second_item.data_ptr(), table.size, table.mean_rate, k.data_ptr(),
                                       u.data_ptr(), _lib.DRAW_UNIT if unit_draws else _lib.DRAW_VALUE, n,
                                       items.data_ptr(), status.data_ptr(), stream), "jfgpu_walker_sample")
    return items[:n].cpu().numpy(), status[:n].cpu().numpy()
