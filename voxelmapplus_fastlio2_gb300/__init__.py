"""GB300-native (sm_103a) FAST-LIO2 + VoxelMapPlus odometry hot path.

The compute lives in _build/libvmp.so (hand-written CUDA, C ABI in
include/vmp.h).  This package holds the host-side mirror of the reference's
LIOBuilder / VoxelMap / IESKF interface (lio.py), the ctypes ABI (abi.py),
the in-tree build (build.py) and the seeded synthetic input generator
(synth.py).
"""
from . import abi  # noqa: F401

__all__ = ["abi", "lio", "synth", "build"]
