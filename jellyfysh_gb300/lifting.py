"""Lifting schemes of composite objects on the GPU: which unit becomes active after an event whose interaction
involves more than two units (``lifting/lifting.py:47-108``).

``select`` decides a batch of tables in one launch through ``jfgpu_lifting`` (``include/jfgpu.h``): the form an
event loop over many chains uses.  ``InsideFirstLifting``, ``OutsideFirstLifting`` and ``RatioLifting`` keep the
reference's interface for one table at a time (``reset`` / ``insert`` / ``get_active_identifier``): they call
Python's ``random.uniform`` exactly where and with the arguments the reference does (so they consume the same random
numbers), raise the reference's exceptions at the same calls, and leave the decision to the GPU.
"""
import random
from typing import Any, List, Sequence, Tuple

import numpy as np

from . import _lib

try:  # the reference's exception when the reference is importable, so that its handlers see their own class
    from jellyfysh.base.exceptions import LiftingSchemeError
except ImportError:  # pragma: no cover - depends on the environment
    class LiftingSchemeError(Exception):
        """Raised when the lifting table holds no active unit (``base/exceptions.py``)."""

SCHEMES = {"inside_first": _lib.LIFTING_INSIDE_FIRST, "outside_first": _lib.LIFTING_OUTSIDE_FIRST,
           "ratio": _lib.LIFTING_RATIO}


def pack(tables: Sequence[Tuple[Sequence[float], Sequence[bool]]]):
    """(rates, active, offsets) arrays of a list of (rates, active) tables, in the layout ``jfgpu_lifting`` reads."""
    counts = np.array([len(r) for r, _ in tables], dtype=np.int64)
    offsets = np.zeros(len(tables) + 1, dtype=np.int64)
    np.cumsum(counts, out=offsets[1:])
    rates = np.zeros(max(int(offsets[-1]), 1), dtype=np.float64)
    active = np.zeros(max(int(offsets[-1]), 1), dtype=np.int32)
    for (r, a), begin, count in zip(tables, offsets[:-1], counts):
        if len(a) != count:
            raise ValueError("every table needs one active flag per derivative")
        rates[begin:begin + count] = r
        active[begin:begin + count] = [1 if x else 0 for x in a]
    return rates, active, offsets


def select(scheme: str, rates, active, offsets, draws, unit_draws: bool = False):
    """Decide n tables in one launch: (selected [n], bound [n], status [n]) as host arrays.

    ``rates`` / ``active`` hold the tables back to back, table i at ``offsets[i]:offsets[i+1]``; ``draws[i]`` is the
    value the deciding ``random.uniform(0.0, b)`` returned, or with ``unit_draws`` the ``random()`` it formed that
    value from.  Arrays may be host arrays or CUDA tensors (used in place)."""
    import torch
    lib = _lib.load()
    device = torch.device("cuda", torch.cuda.current_device())

    def on_device(values, dtype):
        if isinstance(values, torch.Tensor) and values.is_cuda:
            return values.to(dtype).contiguous()
        return torch.as_tensor(np.asarray(values), dtype=dtype).to(device)

    offsets_d = on_device(offsets, torch.int64)
    n = offsets_d.numel() - 1
    if n < 0:
        raise ValueError("offsets needs n + 1 entries")
    rates_d = on_device(rates, torch.float64)
    active_d = on_device(active, torch.int32)
    draws_d = on_device(draws, torch.float64)
    if draws_d.numel() != n:
        raise ValueError("one draw per table")
    if rates_d.numel() == 0:  # the C ABI wants valid pointers even when every table is empty
        rates_d = torch.zeros(1, dtype=torch.float64, device=device)
        active_d = torch.zeros(1, dtype=torch.int32, device=device)
    selected = torch.empty(max(n, 1), dtype=torch.int64, device=device)
    bound = torch.empty(max(n, 1), dtype=torch.float64, device=device)
    status = torch.empty(max(n, 1), dtype=torch.int32, device=device)
    stream = torch.cuda.current_stream(device).cuda_stream
    _lib.check(lib.jfgpu_lifting(SCHEMES[scheme], _lib.DRAW_UNIT if unit_draws else _lib.DRAW_VALUE,
                                 rates_d.data_ptr(), active_d.data_ptr(), offsets_d.data_ptr(), n, draws_d.data_ptr(),
                                 selected.data_ptr(), bound.data_ptr(), status.data_ptr(), stream), "jfgpu_lifting")
    return selected[:n].cpu().numpy(), bound[:n].cpu().numpy(), status[:n].cpu().numpy()


def raise_status(status: int) -> None:
    """Raise the reference's exception for a lifting status (nothing for JFGPU_STATUS_OK)."""
    status = int(status)
    if status == _lib.STATUS_OK:
        return
    if status == _lib.STATUS_LIFTING:
        raise LiftingSchemeError("Active unit has not been recorded.")
    if status == _lib.STATUS_INDEX:
        raise IndexError("list index out of range")
    if status == _lib.STATUS_ASSERTION:
        raise AssertionError("lifting table with a misplaced active unit")
    raise RuntimeError("lifting status %d" % status)


class _GpuLifting:
    """The reference's ``Lifting`` interface (``lifting/lifting.py:38-108``) with the decision on the GPU."""

    scheme = "inside_first"

    def __init__(self) -> None:
        self.reset()

    def reset(self) -> None:
        self._rates: List[float] = []
        self._active: List[bool] = []
        self._identifiers: List[Any] = []
        self._negative_lifting_rates: List[float] = []
        self._draw = 0.0
        self._active_recorded = False

    def insert(self, lifting_rate: float, associated_identifier: Any, is_active: bool) -> None:
        """Insert a factor derivative; the active unit's insert draws random.uniform(0.0, derivative) as the
        reference's does (lifting.py:70-76), a negative derivative of the active unit is an AssertionError."""
        if lifting_rate > 0.0:
            if is_active:
                if self._active_recorded:
                    raise AssertionError("a lifting table holds one active unit")
                self._active_recorded = True
                self._draw = random.uniform(0.0, lifting_rate)
        else:
            assert not is_active
            self._negative_lifting_rates.append(-lifting_rate)
        self._rates.append(float(lifting_rate))
        self._active.append(bool(is_active))
        self._identifiers.append(associated_identifier)

    def _decide(self, draw: float) -> Any:
        rates, active, offsets = pack([(self._rates, self._active)])
        selected, _, status = select(self.scheme, rates, active, offsets, [draw])
        raise_status(status[0])
        return self._identifiers[int(selected[0])]

    def get_active_identifier(self) -> Any:
        if not self._active_recorded:
            raise LiftingSchemeError("Active unit has not been recorded.")
        return self._decide(self._draw)


class InsideFirstLifting(_GpuLifting):
    """``lifting/inside_first_lifting.py:29-54`` on the GPU."""

    scheme = "inside_first"


class OutsideFirstLifting(_GpuLifting):
    """``lifting/outside_first_lifting.py:29-55`` on the GPU."""

    scheme = "outside_first"


class RatioLifting(_GpuLifting):
    """``lifting/ratio_lifting.py:30-56`` on the GPU: draws random.uniform(0.0, sum of the negated negative
    derivatives) in ``get_active_identifier``, as the reference does."""

    scheme = "ratio"

    def get_active_identifier(self) -> Any:
        if not self._active_recorded:
            raise LiftingSchemeError("Active unit has not been recorded.")
        return self._decide(random.uniform(0.0, sum(self._negative_lifting_rates)))
