"""The reference's own CUDA kernels on this GPU.  TEST INFRASTRUCTURE ONLY.

``make -C oracle ref-gpu`` compiles the reference's cuda_functions.cu, from
where it lies in the reference tree, for sm_103a: one device-code-only
cubin per particle count N (oracle/_ref/ref_kernels_n<N>.cubin), because
the reference fixes every size at compile time and recompiles per
configuration (ref_gpu_config.h).  This module loads such a cubin through
the CUDA driver API (ctypes on libcuda) into the context torch uses, and
launches Mss_mult / Mbb_mult exactly as the reference's solver does
(rpy_mobility_solver.cu:241-255, 283-295): ceil(num / 64) blocks of
THREADS_PER_BLOCK = 64 threads, one launch for all targets.

Used by the tests (the reference's GPU results against this library's) and
by ``bench.py --impl reference`` (the reference's GPU time beside its CPU
time).  The product never loads anything from here.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
THREADS_PER_BLOCK = 64
# C++ names of the reference's kernels (cuda_functions.hpp:9-10)
MSS = b"_Z8Mss_multPdPKdS1_ii"
MBB = b"_Z8Mbb_multPdPKdS1_ii"
SEED = b"_Z22seeding_repulsion_stepPdPKdi"


def cubin_path(n: int) -> str:
    return os.path.join(REF_DIR, f"ref_kernels_n{n}.cubin")


def available(n: int) -> bool:
    return os.path.isfile(cubin_path(n))


_cu = None


def _driver():
    global _cu
    if _cu is None:
        lib = ctypes.CDLL("libcuda.so.1")
        lib.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        lib.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        lib.cuModuleUnload.argtypes = [ctypes.c_void_p]
        lib.cuLaunchKernel.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                       ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p,
                                       ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p)]
        lib.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        _cu = lib
    return _cu


def _check(rc: int, what: str) -> None:
    if rc != 0:
        msg = ctypes.c_char_p()
        _driver().cuGetErrorString(rc, ctypes.byref(msg))
        raise RuntimeError(f"{what}: CUDA driver error {rc} ({msg.value.decode() if msg.value else '?'})")


class RefKernels:
    """The reference's kernels built for N particles, loaded into the
    current context (torch's, on the current device)."""

    def __init__(self, n: int):
        import torch
        if not available(n):
            raise FileNotFoundError(f"{cubin_path(n)} is not built (make -C oracle ref-gpu)")
        torch.zeros(1, device="cuda")  # the primary context is current from here on
        self.n = n
        cu = _driver()
        self.mod = ctypes.c_void_p()
        _check(cu.cuModuleLoad(ctypes.byref(self.mod), cubin_path(n).encode()), "cuModuleLoad")
        self.fn = {}
        for key, name in (("mss", MSS), ("mbb", MBB), ("seed", SEED)):
            f = ctypes.c_void_p()
            _check(cu.cuModuleGetFunction(ctypes.byref(f), self.mod, name), f"cuModuleGetFunction {name!r}")
            self.fn[key] = f

    def _launch(self, key, V, F, X, start, num, stream):
        args = [ctypes.c_void_p(V.data_ptr()), ctypes.c_void_p(F.data_ptr()), ctypes.c_void_p(X.data_ptr()),
                ctypes.c_int(start), ctypes.c_int(num)]
        params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        blocks = (num + THREADS_PER_BLOCK - 1) // THREADS_PER_BLOCK
        _check(_driver().cuLaunchKernel(self.fn[key], blocks, 1, 1, THREADS_PER_BLOCK, 1, 1, 0,
                                        ctypes.c_void_p(stream), params, None), f"cuLaunchKernel {key}")

    def mss(self, V, F, X, start=0, num=None, stream=None):
        """V = M_ss F for segments [start, start + num) of the N built in
        (float64 CUDA tensors: V (num, 6), F (N, 6), X (N, 3))."""
        import torch
        num = self.n - start if num is None else num
        s = torch.cuda.current_stream().cuda_stream if stream is None else stream
        self._launch("mss", V, F, X, start, num, s)

    def mbb(self, V, F, X, start=0, num=None, stream=None):
        import torch
        num = self.n - start if num is None else num
        s = torch.cuda.current_stream().cuda_stream if stream is None else stream
        self._launch("mbb", V, F, X, start, num, s)

    def seed_sphere(self, n, max_steps=100000):
        """The reference's repulsive seeding of n points (seeding.cu:13-160,
        its GPU path): the spiral start on the host, then per step the
        reference's seeding_repulsion_step kernel for the forces and the
        host update of seeding.cu:113-136 (numpy, elementwise in the written
        order).  Returns (points (n, 3), steps)."""
        import math

        import numpy as np
        import torch
        x = np.zeros((n, 3))
        phi = 0.0
        for m in range(n):
            z = -1.0 if n == 1 else 2.0 * m / float(n - 1) - 1.0
            r = math.sqrt(1.0 - z * z)
            if m == 0 or m == n - 1:
                phi = 0.0
            else:
                phi += 3.6 / (r * math.sqrt(n))
            x[m] = (r * math.cos(phi), r * math.sin(phi), z)
        X = torch.empty((n, 3), dtype=torch.float64, device="cuda")
        F = torch.empty((n, 3), dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        blocks = (n + THREADS_PER_BLOCK - 1) // THREADS_PER_BLOCK
        steps = 0
        while steps < max_steps:
            X.copy_(torch.as_tensor(x))
            args = [ctypes.c_void_p(F.data_ptr()), ctypes.c_void_p(X.data_ptr()), ctypes.c_int(n)]
            params = (ctypes.c_void_p * 3)(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
            _check(_driver().cuLaunchKernel(self.fn["seed"], blocks, 1, 1, THREADS_PER_BLOCK, 1, 1, 0,
                                            ctypes.c_void_p(stream), params, None), "cuLaunchKernel seed")
            f = F.cpu().numpy()
            p = x + f
            nrm = np.sqrt(p[:, 0] * p[:, 0] + p[:, 1] * p[:, 1] + p[:, 2] * p[:, 2])
            p = p / nrm[:, None]
            move = float(np.abs(p - x).max())
            x = p
            steps += 1
            if move <= 1e-4:
                break
        return x, steps

    def close(self):
        if getattr(self, "mod", None):
            _driver().cuModuleUnload(self.mod)
            self.mod = None
