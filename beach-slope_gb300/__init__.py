"""beachslope_gb300 -- host side of the GB300 ISPH particle hot path.

The compute path is libbeachslope.so (hand-written sm_103a CUDA behind the
C-ABI in include/beachslope.h).  This package only holds the ctypes mirror of
that ABI, the host-side context wrapper and the synthetic scene generators.
There is no CPU fallback: importing `api` without the built library raises.
"""
from . import abi, scene  # noqa: F401

__all__ = ["abi", "scene", "api", "build"]
