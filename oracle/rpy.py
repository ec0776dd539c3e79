"""ctypes front end of the FP64 CPU oracle (rpy_oracle.c) and of the reference's
own kernels compiled for the CPU (oracle/_ref).  TEST INFRASTRUCTURE ONLY.

Every function takes and returns numpy float64 arrays in the reference's
host layouts: positions (n, 3), segment forces/torques (S, 6) ordered
(f, tau), blob forces (B, 3); segment velocities come back as (S, 6)
ordered (v, omega) and blob velocities as (B, 3).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from functools import lru_cache

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORC_SO = os.path.join(HERE, "_build", "liborc.so")
REF_DIR = os.path.join(HERE, "_ref")

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.c_int
_F = ctypes.c_double


def build(with_reference: bool | None = None) -> None:
    """Compile the restatement (always) and, when the reference tree is
    present, the reference's own kernels for the CPU."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    from oracle import reference_dir
    ref_root = reference_dir()
    if with_reference is None:
        with_reference = os.path.isfile(os.path.join(ref_root, "cuda_functions.cu"))
    if with_reference:
        subprocess.run(["make", "-s", "-j4", "-C", HERE, "ref", "ref-gpu", f"REF={ref_root}"], check=True)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _c64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


@lru_cache(maxsize=None)
def _orc() -> ctypes.CDLL:
    if not os.path.exists(ORC_SO):
        build(with_reference=False)
    lib = ctypes.CDLL(ORC_SO)
    lib.orc_mss.argtypes = [_I, _D, _D, _F, _F, _I, _I, _D]
    lib.orc_mss_wall.argtypes = [_I, _D, _D, _I, _I, _D]
    lib.orc_mbb.argtypes = [_I, _D, _D, _F, _F, _I, _I, _D]
    lib.orc_msb.argtypes = [_I, _I, _D, _D, _D, _F, _F, _F, _I, _I, _D]
    lib.orc_mbs.argtypes = [_I, _I, _D, _D, _D, _F, _F, _F, _I, _I, _D]
    lib.orc_barrier.argtypes = [_I, _I, _I, _D, _D, _F, _F, _F, _I, _D, _D]
    for f in (lib.orc_mss, lib.orc_mss_wall, lib.orc_mbb, lib.orc_msb, lib.orc_mbs, lib.orc_barrier):
        f.restype = None
    return lib


def _range(n: int, targets):
    if targets is None:
        return 0, n
    t0, nt = targets
    assert 0 <= t0 and nt >= 0 and t0 + nt <= n
    return t0, nt


def mss(xs, fs, a=1.0, mu=1.0, targets=None):
    """Segment<-segment free-space RPY (cuda_functions.cu:246-425)."""
    xs, fs = _c64(xs), _c64(fs)
    S = xs.shape[0]
    t0, nt = _range(S, targets)
    out = np.empty((nt, 6))
    _orc().orc_mss(S, _ptr(xs), _ptr(fs), a, mu, t0, nt, _ptr(out))
    return out


def mss_wall(xs, fs, targets=None):
    """Segment<-segment above a no-slip wall, a = mu = 1 (cuda_functions.cu:10-242)."""
    xs, fs = _c64(xs), _c64(fs)
    S = xs.shape[0]
    t0, nt = _range(S, targets)
    out = np.empty((nt, 6))
    _orc().orc_mss_wall(S, _ptr(xs), _ptr(fs), t0, nt, _ptr(out))
    return out


def mbb(xb, fb, a=1.0, mu=1.0, targets=None):
    """Blob<-blob RPY (cuda_functions.cu:429-539)."""
    xb, fb = _c64(xb), _c64(fb)
    B = xb.shape[0]
    t0, nt = _range(B, targets)
    out = np.empty((nt, 3))
    _orc().orc_mbb(B, _ptr(xb), _ptr(fb), a, mu, t0, nt, _ptr(out))
    return out


def msb(xs, xb, fb, a_seg=1.0, a_blob=1.0, mu=1.0, v_in=None):
    """Segment<-blob RPY; accumulates onto v_in (cuda_functions.cu:541-694)."""
    xs, xb, fb = _c64(xs), _c64(xb), _c64(fb)
    S, B = xs.shape[0], xb.shape[0]
    out = np.zeros((S, 6)) if v_in is None else _c64(v_in).copy()
    _orc().orc_msb(S, B, _ptr(xs), _ptr(xb), _ptr(fb), a_seg, a_blob, mu, 0, S, _ptr(out))
    return out


def mbs(xb, xs, fs, a_seg=1.0, a_blob=1.0, mu=1.0):
    """Blob<-segment RPY; overwrites (cuda_functions.cu:697-863)."""
    xb, xs, fs = _c64(xb), _c64(xs), _c64(fs)
    S, B = xs.shape[0], xb.shape[0]
    out = np.empty((B, 3))
    _orc().orc_mbs(B, S, _ptr(xb), _ptr(xs), _ptr(fs), a_seg, a_blob, mu, 0, B, _ptr(out))
    return out


def barrier(xs, xb, fs, nseg, a_seg=1.0, a_blob=1.0, scale=1.0, wall=False):
    """Barrier forces (cuda_functions.cu:961-1157).  Returns (fs + segment
    repulsion, blob repulsion)."""
    xs, xb = _c64(xs), _c64(xb).reshape(-1, 3)
    fs_out = _c64(fs).copy()
    S, B = xs.shape[0], xb.shape[0]
    fb = np.zeros((B, 3))
    _orc().orc_barrier(S, B, nseg, _ptr(xs), _ptr(xb), a_seg, a_blob, scale, int(wall),
                       _ptr(fs_out), _ptr(fb))
    return fs_out, fb


# --------------------------------------------------------------------------
# The reference's own kernels compiled for the CPU (present only where the
# reference tree was available at build time).
# --------------------------------------------------------------------------
def have_reference_kernels() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libref_kernels_free.so"))


@lru_cache(maxsize=None)
def _ref(wall: bool) -> ctypes.CDLL:
    path = os.path.join(REF_DIR, "libref_kernels_wall.so" if wall else "libref_kernels_free.so")
    lib = ctypes.CDLL(path)
    lib.ref_set_problem.argtypes = [_I, _I, _I, _I, _F, _F, _F, _F, _F]
    lib.ref_mss.argtypes = [_D, _D, _D]
    lib.ref_mbb.argtypes = [_D, _D, _D]
    lib.ref_msb.argtypes = [_D, _D, _D, _D]
    lib.ref_mbs.argtypes = [_D, _D, _D, _D]
    lib.ref_barrier.argtypes = [_D, _D, _D, _D]
    return lib


class RefKernels:
    """The reference's kernels for one problem: nfil filaments of nseg
    segments and nblob blobs per swimmer, nswim swimmers."""

    def __init__(self, nswim, nfil, nseg, nblob, rseg=1.0, rblob=1.0, mu=1.0,
                 repulsive_force_factor=1.0, end_force_magnitude=1.0, wall=False):
        self.lib = _ref(wall)
        self.S = nswim * nfil * nseg
        self.B = nswim * nblob
        self.args = (nswim, nfil, nseg, nblob, rseg, rblob, mu,
                     repulsive_force_factor, end_force_magnitude)

    def _set(self):
        self.lib.ref_set_problem(*self.args)

    def mss(self, xs, fs):
        xs, fs = _c64(xs), _c64(fs)
        out = np.empty((self.S, 6))
        self._set()
        self.lib.ref_mss(_ptr(out), _ptr(fs), _ptr(xs))
        return out

    def mbb(self, xb, fb):
        xb, fb = _c64(xb), _c64(fb)
        out = np.empty((self.B, 3))
        self._set()
        self.lib.ref_mbb(_ptr(out), _ptr(fb), _ptr(xb))
        return out

    def msb(self, xs, xb, fb, v_in):
        xs, xb, fb = _c64(xs), _c64(xb), _c64(fb)
        out = _c64(v_in).copy()
        self._set()
        self.lib.ref_msb(_ptr(out), _ptr(fb), _ptr(xs), _ptr(xb))
        return out

    def mbs(self, xb, xs, fs):
        xb, xs, fs = _c64(xb), _c64(xs), _c64(fs)
        out = np.empty((self.B, 3))
        self._set()
        self.lib.ref_mbs(_ptr(out), _ptr(fs), _ptr(xb), _ptr(xs))
        return out

    def barrier(self, xs, xb, fs):
        xs = _c64(xs)
        xb = _c64(xb).reshape(-1, 3)
        fs_out = _c64(fs).copy()
        fb = np.zeros((max(self.B, 1), 3))
        xb_arg = xb if xb.size else np.zeros((1, 3))
        self._set()
        self.lib.ref_barrier(_ptr(fs_out), _ptr(fb), _ptr(xs), _ptr(xb_arg))
        return fs_out, fb[: self.B]
