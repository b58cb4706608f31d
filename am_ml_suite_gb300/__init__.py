"""GB300-native (sm_103a) SIMP topology-optimisation engine.

The compute path is the native library ``lib/libamgpu.so`` (hand-written CUDA
behind the C ABI of ``include/am_gpu.h``); ``_native`` binds it with ctypes,
``numerical`` mirrors the reference's Python numerical path, ``cpp`` the
Python surface of its C++ engine, ``core`` the problem-definition types.
"""
from . import _native
from ._native import AmError, Problem, default_config, is_available

__all__ = ["AmError", "Problem", "default_config", "is_available", "_native"]
