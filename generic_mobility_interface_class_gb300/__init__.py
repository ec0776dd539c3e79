"""GB300-native RPY mobility apply and the GMRES/Broyden solves that consume it.

The compute path is libgmi.so (hand-written CUDA for sm_103a behind the C ABI
declared in include/gmi.h).  This package holds its build script, its ctypes
binding and thin host-side helpers; PyTorch is used only to own device
memory in tests and benchmarks.
"""
from ._lib import GMI_DF64, GMI_FP32C, GMI_FP64, GmiError, GmiLibraryMissing  # noqa: F401

__all__ = ["GMI_FP64", "GMI_FP32C", "GMI_DF64", "GmiError", "GmiLibraryMissing"]
