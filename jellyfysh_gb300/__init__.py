"""GB300-native event-time engine for event-chain Monte Carlo, with JeLLyFysh's interfaces.

The compute path is ``libjfgpu.so`` (hand-written CUDA for sm_103a, C ABI in ``include/jfgpu.h``); this package is
its host side: ctypes bindings (``_lib``), the batched chain engine (``chains``), GPU potentials with the reference's
``displacement`` / ``derivative`` interface (``potential``) and seeded synthetic initial states (``systems``).
"""
from . import _lib  # noqa: F401
from .chains import ChainBatch, ChainSpec, chain_key  # noqa: F401

__all__ = ["ChainBatch", "ChainSpec", "chain_key"]
