"""ctypes binding of libgmi.so (include/gmi.h).

The library must have been built (``build.build()``); there is no fallback:
importing a function from a missing library raises GmiLibraryMissing.
"""
from __future__ import annotations

import ctypes
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "_build", "libgmi.so")
HEADER = os.path.join(ROOT, "include", "gmi.h")

GMI_OK = 0
GMI_FP64 = 0
GMI_FP32C = 1
STATUS_NAMES = {0: "GMI_OK", 1: "GMI_ERR_ARG", 2: "GMI_ERR_CUDA", 3: "GMI_ERR_DEVICE_TIMEOUT",
                4: "GMI_ERR_NONFINITE", 5: "GMI_ERR_NOT_CONVERGED", 6: "GMI_ERR_STATE"}


class GmiLibraryMissing(RuntimeError):
    pass


class GmiError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double

# argument types of every exported function, in header order
SIGNATURES = {
    "gmi_last_error": ([], ctypes.c_char_p),
    "gmi_version": ([], _I),
    "gmi_context_create": ([_I, ctypes.POINTER(_P)], _I),
    "gmi_context_destroy": ([_P], _I),
    "gmi_context_set_stream": ([_P, _P], _I),
    "gmi_context_set_precision": ([_P, _I], _I),
    "gmi_context_precision": ([_P], _I),
    "gmi_context_synchronize": ([_P], _I),
    "gmi_context_launch_count": ([_P], ctypes.c_longlong),
    "gmi_Mss_mult": ([_P, _P, _P, _P, _I, _I, _I, _D, _D], _I),
    "gmi_Mss_mult_wall": ([_P, _P, _P, _P, _I, _I, _I], _I),
    "gmi_Mbb_mult": ([_P, _P, _P, _P, _I, _I, _I, _D, _D], _I),
    "gmi_Msb_mult": ([_P, _P, _P, _P, _P, _I, _I, _I, _I, _D, _D, _D], _I),
    "gmi_Mbs_mult": ([_P, _P, _P, _P, _P, _I, _I, _I, _I, _D, _D, _D], _I),
    "gmi_barrier_forces": ([_P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _I, _D, _D, _D, _I], _I),
    "gmi_autotune": ([_P, _I, _I, _I], _I),
    "gmi_measure_fma_peak": ([_P, _I, ctypes.POINTER(_D)], _I),
}

_lib = None


def header_symbols() -> list[str]:
    """Names of the functions include/gmi.h declares."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"GMI_API\s+[\w\s\*]*?\b(gmi_\w+)\s*\(", text)))


def load() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise GmiLibraryMissing(
            f"{LIB_PATH} is not built; run generic_mobility_interface_class_gb300.build.build() first")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != GMI_OK:
        msg = load().gmi_last_error()
        raise GmiError(status, msg.decode() if msg else "")
