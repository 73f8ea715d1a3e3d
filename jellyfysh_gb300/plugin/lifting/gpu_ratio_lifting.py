"""Factory name ``gpu_ratio_lifting``: the reference's ``RatioLifting`` (``lifting/ratio_lifting.py:30-56``), decided on the GPU."""
from jellyfysh_gb300.lifting import RatioLifting


class GpuRatioLifting(RatioLifting):
    """Drop-in for ``RatioLifting`` in an event handler's ``lifting`` option."""
