"""Host-side Python wrapper of the gmi_context pair sums (include/gmi.h).

Arrays are torch tensors on the context's GPU, float64, in the reference's
AoS layouts: positions (n, 3), segment forces/torques (S, 6), blob forces
(B, 3).  The context runs on torch's current CUDA stream, so torch work and
library kernels are ordered without extra synchronisation.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import GMI_FP32C, GMI_FP64, check

KIND_SS, KIND_SS_WALL, KIND_BB, KIND_SB, KIND_BS = range(5)


def _dev(t: torch.Tensor, rows: int, cols: int, name: str) -> int:
    if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
        raise ValueError(f"{name} must be a contiguous float64 CUDA tensor")
    if t.numel() != rows * cols:
        raise ValueError(f"{name} must hold {rows}x{cols} values, got {tuple(t.shape)}")
    return t.data_ptr()


class Context:
    """One GPU context of libgmi (gmi_context_*)."""

    def __init__(self, device: int = 0, precision: int = GMI_FP64, stream: torch.cuda.Stream | None = None):
        self.lib = _lib.load()
        self.device = device
        h = ctypes.c_void_p()
        check(self.lib.gmi_context_create(device, ctypes.byref(h)))
        self.handle = h
        s = stream if stream is not None else torch.cuda.current_stream(device)
        # torch's default stream has handle 0; the library needs the explicit
        # cudaStreamLegacy handle (1) for it, since NULL means "own stream".
        check(self.lib.gmi_context_set_stream(self.handle, ctypes.c_void_p(s.cuda_stream or 1)))
        self.set_precision(precision)

    def set_precision(self, precision: int) -> None:
        check(self.lib.gmi_context_set_precision(self.handle, precision))
        self.precision = precision

    def synchronize(self) -> None:
        check(self.lib.gmi_context_synchronize(self.handle))

    @property
    def launches(self) -> int:
        return int(self.lib.gmi_context_launch_count(self.handle))

    def set_wait_deadline(self, nanoseconds: int) -> None:
        """Deadline of the pair kernels' bounded waits (0: the 2 s default)."""
        check(self.lib.gmi_context_set_wait_deadline(self.handle, int(nanoseconds)))

    def check_bounded_wait(self, withhold_arrival: bool) -> None:
        """Run the bounded-wait check kernel; raises GmiError
        (GMI_ERR_DEVICE_TIMEOUT) when an arrival is withheld."""
        check(self.lib.gmi_context_check_bounded_wait(self.handle, int(withhold_arrival)))

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.gmi_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- pair sums (reference kernels cuda_functions.cu:10-863) ----------
    def mss(self, xs, fs, a=1.0, mu=1.0, start=0, num=None, out=None):
        S = xs.shape[0]
        num = S - start if num is None else num
        out = torch.empty((num, 6), dtype=torch.float64, device=xs.device) if out is None else out
        check(self.lib.gmi_Mss_mult(self.handle, _dev(out, num, 6, "V"), _dev(fs, S, 6, "F"),
                                    _dev(xs, S, 3, "X"), start, num, S, a, mu))
        return out

    def mss_wall(self, xs, fs, start=0, num=None, out=None):
        S = xs.shape[0]
        num = S - start if num is None else num
        out = torch.empty((num, 6), dtype=torch.float64, device=xs.device) if out is None else out
        check(self.lib.gmi_Mss_mult_wall(self.handle, _dev(out, num, 6, "V"), _dev(fs, S, 6, "F"),
                                         _dev(xs, S, 3, "X"), start, num, S))
        return out

    def mbb(self, xb, fb, a=1.0, mu=1.0, start=0, num=None, out=None):
        B = xb.shape[0]
        num = B - start if num is None else num
        out = torch.empty((num, 3), dtype=torch.float64, device=xb.device) if out is None else out
        check(self.lib.gmi_Mbb_mult(self.handle, _dev(out, num, 3, "V"), _dev(fb, B, 3, "F"),
                                    _dev(xb, B, 3, "X"), start, num, B, a, mu))
        return out

    def msb(self, xs, xb, fb, v_inout, a_seg=1.0, a_blob=1.0, mu=1.0, start=0, num=None):
        """v_inout += M_sb fb (in place), as the reference's Msb_mult."""
        S, B = xs.shape[0], xb.shape[0]
        num = S - start if num is None else num
        check(self.lib.gmi_Msb_mult(self.handle, _dev(v_inout, num, 6, "V"), _dev(fb, B, 3, "F"),
                                    _dev(xs, S, 3, "Xs"), _dev(xb, B, 3, "Xb"), start, num, S, B,
                                    a_seg, a_blob, mu))
        return v_inout

    def mbs(self, xb, xs, fs, a_seg=1.0, a_blob=1.0, mu=1.0, start=0, num=None, out=None):
        S, B = xs.shape[0], xb.shape[0]
        num = B - start if num is None else num
        out = torch.empty((num, 3), dtype=torch.float64, device=xb.device) if out is None else out
        check(self.lib.gmi_Mbs_mult(self.handle, _dev(out, num, 3, "V"), _dev(fs, S, 6, "F"),
                                    _dev(xb, B, 3, "Xb"), _dev(xs, S, 3, "Xs"), start, num, B, S,
                                    a_seg, a_blob, mu))
        return out

    def barrier(self, xs, xb, fs_inout, nseg, a_seg=1.0, a_blob=1.0, scale=1.0, wall=False, fb_out=None):
        """fs_inout[:, :3] += segment repulsion (in place); returns blob repulsion."""
        S, B = xs.shape[0], xb.shape[0]
        if fb_out is None:
            fb_out = torch.zeros((max(B, 1), 3), dtype=torch.float64, device=xs.device)
        check(self.lib.gmi_barrier_forces(
            self.handle, _dev(fs_inout, S, 6, "f_segs") if S else None,
            fb_out.data_ptr() if B else None,
            _dev(xs, S, 3, "x_segs") if S else None, _dev(xb, B, 3, "x_blobs") if B else None,
            0, S, 0, B, S, B, nseg, a_seg, a_blob, scale, int(wall)))
        return fb_out[:B]

    def fma_peak(self, precision: int) -> float:
        """Measured FMA-pipe FLOP/s of this GPU (FMA = 2 FLOP)."""
        out = ctypes.c_double()
        check(self.lib.gmi_measure_fma_peak(self.handle, precision, ctypes.byref(out)))
        return out.value

    def autotune(self, kind: int, num_targets: int, num_sources: int) -> None:
        check(self.lib.gmi_autotune(self.handle, kind, num_targets, num_sources))

    def tuned_shape(self, kind: int, num_targets: int, num_sources: int):
        """(threads per CTA, targets per thread, source splits, tuned?)."""
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        st = self.lib.gmi_tuned_shape(self.handle, kind, num_targets, num_sources, ctypes.byref(a),
                                      ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value, st == 0

    def tuned_sources_per_step(self, kind: int, num_targets: int, num_sources: int) -> int:
        """2 when that size runs the packed FP32 kernel (two sources per
        f32x2 step), else 1."""
        a = ctypes.c_int()
        self.lib.gmi_tuned_sources_per_step(self.handle, kind, num_targets, num_sources, ctypes.byref(a))
        return a.value

    def set_shape(self, kind: int, num_targets: int, num_sources: int, threads_per_cta: int,
                  targets_per_thread: int, source_splits: int = 0, sources_per_step: int = 2) -> None:
        """Pin the launch shape used for this kernel and size."""
        check(self.lib.gmi_set_shape(self.handle, kind, num_targets, num_sources, threads_per_cta,
                                     targets_per_thread, source_splits, sources_per_step))
