"""GB300-native XPBD soft-body solver: Python surface over libvsim.

The compute path is libvsim.so (hand-written sm_103a CUDA kernels behind a
C ABI, include/vsim.h); this package binds it with ctypes, mirrors the
reference's `Simulator` class, and generates the synthetic workloads.
"""
from ._ffi import VsimError, VsimRangeError, lib  # noqa: F401
from .scenes import Scene, Body  # noqa: F401
from .simulator import Simulator  # noqa: F401
