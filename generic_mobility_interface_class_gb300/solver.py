"""Python wrapper of the device-resident mobility solver (gmi_solver_*).

Mirrors the reference's mobility_solver / rpy_mobility_solver interface
(mobility_solver.hpp:18-102): the solver owns pinned host arrays that the
caller fills in place (x_segs_host, f_segs_host, ...), exposed here as numpy
views, and the per-backend operations keep the reference's names.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import GMI_FP64, HostArrays, SolverConfig, check


def _view(ptr, count, cols):
    if count == 0:
        return np.zeros((0, cols))
    return np.ctypeslib.as_array(ptr, shape=(count * cols,)).reshape(count, cols)


def _cptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class MobilitySolver:
    """gmi_solver: nswim swimmers x (nblob blobs, nfil filaments x nseg segments)."""

    def __init__(self, nswim=1, nfil=0, nseg=1, nblob=0, mu=1.0, rseg=1.0, rblob=1.0,
                 repulsive_force_factor=2.0, end_force_magnitude=1.0, wall=False, max_linear_iter=150,
                 linear_tol=1e-10, precision=GMI_FP64, device=0):
        self.lib = _lib.load()
        cfg = SolverConfig(nswim, nfil, nseg, nblob, mu, rseg, rblob, repulsive_force_factor, end_force_magnitude,
                           int(wall), max_linear_iter, linear_tol, precision, device)
        self.cfg = cfg
        h = ctypes.c_void_p()
        check(self.lib.gmi_solver_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h
        arrays = HostArrays()
        check(self.lib.gmi_solver_host_arrays(self.handle, ctypes.byref(arrays)))
        S, B = nswim * nfil * nseg, nswim * nblob
        self.S, self.B, self.W = S, B, nswim
        self.v_segs_host = _view(arrays.v_segs_host, S, 6)
        self.v_blobs_host = _view(arrays.v_blobs_host, B, 3)
        self.x_segs_host = _view(arrays.x_segs_host, S, 3)
        self.x_blobs_host = _view(arrays.x_blobs_host, B, 3)
        self.f_segs_host = _view(arrays.f_segs_host, S, 6)
        self.f_blobs_host = _view(arrays.f_blobs_host, B, 3)
        self.f_blobs_repulsion_host = _view(arrays.f_blobs_repulsion_host, B, 3)

    # ---- lifetime ----------------------------------------------------------
    def close(self):
        if getattr(self, "handle", None):
            self.lib.gmi_solver_destroy(self.handle)
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

    @property
    def launches(self) -> int:
        return int(self.lib.gmi_context_launch_count(self.lib.gmi_solver_context(self.handle)))

    # ---- the per-backend operations (mobility_solver.hpp:25-44) ---------------
    def _call(self, name):
        check(getattr(self.lib, "gmi_solver_" + name)(self.handle))

    def copy_segment_positions_to_device(self): self._call("copy_segment_positions_to_device")
    def copy_segment_forces_to_device(self): self._call("copy_segment_forces_to_device")
    def copy_blob_positions_to_device(self): self._call("copy_blob_positions_to_device")
    def copy_blob_forces_to_device(self): self._call("copy_blob_forces_to_device")
    def copy_interparticle_blob_forces_to_host(self): self._call("copy_interparticle_blob_forces_to_host")
    def copy_blob_velocities_to_host(self): self._call("copy_blob_velocities_to_host")
    def copy_segment_velocities_to_host(self): self._call("copy_segment_velocities_to_host")
    def apply_interparticle_forces(self): self._call("apply_interparticle_forces")
    def wait_for_device(self): self._call("wait_for_device")
    def evaluate_segment_segment_mobility(self): self._call("evaluate_segment_segment_mobility")
    def evaluate_segment_blob_mobility(self): self._call("evaluate_segment_blob_mobility")
    def evaluate_blob_blob_mobility(self): self._call("evaluate_blob_blob_mobility")
    def evaluate_blob_segment_mobility(self): self._call("evaluate_blob_segment_mobility")

    # ---- generic methods, device resident -------------------------------------
    def set_blob_references(self, refs):
        refs = np.ascontiguousarray(refs, dtype=np.float64)
        check(self.lib.gmi_solver_set_blob_references(self.handle, _cptr(refs)))

    def make_body_reference_matrices(self, body_x, body_q):
        bx = np.ascontiguousarray(body_x, dtype=np.float64)
        bq = np.ascontiguousarray(body_q, dtype=np.float64)
        ktk = np.zeros(36)
        mob = np.zeros(36)
        check(self.lib.gmi_solver_make_body_reference_matrices(self.handle, _cptr(bx), _cptr(bq), _cptr(ktk),
                                                               _cptr(mob)))
        return ktk.reshape(6, 6, order="F"), mob.reshape(6, 6, order="F")

    def set_body_reference_matrices(self, ktkinv, mob):
        a = np.asfortranarray(ktkinv, dtype=np.float64).ravel(order="F")
        b = np.asfortranarray(mob, dtype=np.float64).ravel(order="F")
        check(self.lib.gmi_solver_set_body_reference_matrices(self.handle, _cptr(a), _cptr(b)))

    def compute_velocities(self, body_x=None, body_q=None, body_f=None):
        """Returns (number of GMRES iterations, body_f after adding the blob
        repulsion).  Inputs are read from x_segs_host / f_segs_host."""
        W = self.W
        bx = np.ascontiguousarray(np.zeros((W, 3)) if body_x is None else body_x, dtype=np.float64)
        bq = np.ascontiguousarray(np.tile([1.0, 0, 0, 0], (W, 1)) if body_q is None else body_q, dtype=np.float64)
        bf = np.array(np.zeros((W, 6)) if body_f is None else body_f, dtype=np.float64, order="C")
        it = ctypes.c_int()
        check(self.lib.gmi_solver_compute_velocities(self.handle, _cptr(bx), _cptr(bq), _cptr(bf), ctypes.byref(it)))
        return it.value, bf

    def compute_velocities_prescribed(self, vel_dir, phase_speed, body_x=None, body_q=None):
        """Prescribed-shape cilia: returns the number of GMRES iterations; the
        segment forces land in f_segs_host[:, :3], the blob forces in
        f_blobs_host, the body velocities in v_bodies().  Segment positions are
        read from x_segs_host; vel_dir is (S, 3), phase_speed (W*nfil,)."""
        W = self.W
        bx = np.ascontiguousarray(np.zeros((W, 3)) if body_x is None else body_x, dtype=np.float64)
        bq = np.ascontiguousarray(np.tile([1.0, 0, 0, 0], (W, 1)) if body_q is None else body_q, dtype=np.float64)
        vd = np.ascontiguousarray(vel_dir, dtype=np.float64)
        ph = np.ascontiguousarray(phase_speed, dtype=np.float64)
        it = ctypes.c_int()
        check(self.lib.gmi_solver_compute_velocities_prescribed(self.handle, _cptr(bx), _cptr(bq), _cptr(vd), _cptr(ph),
                                                                ctypes.byref(it)))
        return it.value

    def set_generalised_force_refs(self, refs) -> None:
        """The beat's generalised-force table over one period (count >= 2
        samples; empty clears it), as the reference reads it from its
        reference file (mobility_solver.cpp:37-65)."""
        r = np.ascontiguousarray(refs, dtype=np.float64).ravel()
        check(self.lib.gmi_solver_set_generalised_force_refs(self.handle, _cptr(r) if r.size else None, int(r.size)))

    def compute_velocities_prescribed_dynamic(self, vel_dir, phase, omega0, phase_speed=None, body_x=None,
                                              body_q=None):
        """Prescribed-shape cilia with the phase speeds solved for
        (DYNAMIC_PHASE_EVOLUTION).  phase, omega0: (W*nfil,) phases and
        natural frequencies; phase_speed: the initial guess (default omega0,
        as the reference).  Returns (GMRES iterations, phase speeds); the
        forces and body velocities land as in compute_velocities_prescribed."""
        W = self.W
        bx = np.ascontiguousarray(np.zeros((W, 3)) if body_x is None else body_x, dtype=np.float64)
        bq = np.ascontiguousarray(np.tile([1.0, 0, 0, 0], (W, 1)) if body_q is None else body_q, dtype=np.float64)
        vd = np.ascontiguousarray(vel_dir, dtype=np.float64)
        ph = np.ascontiguousarray(phase, dtype=np.float64)
        om = np.ascontiguousarray(omega0, dtype=np.float64)
        sp = np.array(om if phase_speed is None else phase_speed, dtype=np.float64).ravel()
        if vd.size != 3 * self.S or ph.size != sp.size or om.size != sp.size or sp.size != W * self.cfg.nfil:
            raise ValueError("vel_dir must hold 3 values per segment; phase, omega0, phase_speed one per filament")
        it = ctypes.c_int()
        check(self.lib.gmi_solver_compute_velocities_prescribed_dynamic(
            self.handle, _cptr(bx), _cptr(bq), _cptr(vd), _cptr(ph), _cptr(om), _cptr(sp), ctypes.byref(it)))
        return it.value, sp

    def last_linear_solve(self):
        """(GMRES iterations, relative residual) of the last linear solve."""
        it, res = ctypes.c_int(), ctypes.c_double()
        check(self.lib.gmi_solver_last_linear_solve(self.handle, ctypes.byref(it), ctypes.byref(res)))
        return it.value, res.value

    def set_strict_convergence(self, strict: bool) -> None:
        """Report a linear solve that stops at its cap above tolerance as
        GMI_ERR_NOT_CONVERGED (the reference accepts it silently)."""
        check(self.lib.gmi_solver_set_strict_convergence(self.handle, int(strict)))

    def v_bodies(self):
        out = np.zeros((self.W, 6))
        check(self.lib.gmi_solver_get_v_bodies(self.handle, _cptr(out)))
        return out

    def set_v_bodies(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        check(self.lib.gmi_solver_set_v_bodies(self.handle, _cptr(v)))
