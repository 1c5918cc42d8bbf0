"""GB300-native block sorting (forward / inverse BWT) for qz's BSC stage.

The compute path is libqzgpu.so (hand-written sm_103a CUDA behind a C ABI,
include/qzgpu.h); this package holds its build recipe, a ctypes binding, and
seeded synthetic workloads with the shapes of qz's streams.
"""
from .native import QzGpuError  # noqa: F401

__all__ = ["QzGpuError"]
