"""Factory name ``gpu_outside_first_lifting``: the reference's ``OutsideFirstLifting`` (``lifting/outside_first_lifting.py:29-55``), decided on the GPU."""
from jellyfysh_gb300.lifting import OutsideFirstLifting


class GpuOutsideFirstLifting(OutsideFirstLifting):
    """Drop-in for ``OutsideFirstLifting`` in an event handler's ``lifting`` option."""
