"""Factory name ``gpu_inside_first_lifting``: the reference's ``InsideFirstLifting`` (``lifting/inside_first_lifting.py:29-54``), decided on the GPU."""
from jellyfysh_gb300.lifting import InsideFirstLifting


class GpuInsideFirstLifting(InsideFirstLifting):
    """Drop-in for ``InsideFirstLifting`` in an event handler's ``lifting`` option."""
