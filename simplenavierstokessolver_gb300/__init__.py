"""GB300-native (sm_103a) SMR-RK3 time step of NaokiHori/SimpleNavierStokesSolver.

The product is ``_lib/libsns_gpu.so`` (C ABI in ``include/sns_gpu.h``); this
package holds its CUDA/C++ sources (``csrc/``), the build recipe and a thin
Python mirror of the reference's operator interface for tests and benchmarks.
"""
from .solver import Case, kernel_launches  # noqa: F401
from ._native import SnsError, lib  # noqa: F401

__all__ = ["Case", "SnsError", "kernel_launches", "lib"]
