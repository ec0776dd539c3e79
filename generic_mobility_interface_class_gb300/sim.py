"""Python wrapper of the device time step (gmi_sim_*): the reference's main
loop (cilia_sim_main.cpp:205-343) for free-swimming spherical swimmers."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib, formats
from ._lib import GMI_FP64, SimConfig, SolverConfig, check

STATE = dict(seg_x=(0, 3), seg_q=(1, 4), seg_u=(2, 3), seg_v=(3, 6), seg_f=(4, 6), body_x=(5, 3), body_q=(6, 4),
             body_u=(7, 3), body_v=(8, 6), lam=(9, 3), tether=(10, 3), clamp=(11, 3), blob_f=(12, 3),
             seg_f_internal=(13, 6))


def _c(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(ctypes.c_void_p)


class Simulation:
    def __init__(self, *, nswim=1, nfil, nseg, nblob, blob_refs, fil_refs, body_x0=None, perturbation1=None,
                 perturbation2=None, mu=1.0, rseg=1.0, rblob=1.0, kb, kt, dt, end_force_magnitude,
                 repulsive_force_factor=2.0, body_radius, tol=1e-4, max_broyden_iter=100, jacobian_confidence=0.1,
                 num_euler_steps=1, linear_tol=1e-10, max_linear_iter=150, precision=GMI_FP64, device=0,
                 wall=False, beat=None):
        self.lib = _lib.load()
        mob = SolverConfig(nswim, nfil, nseg, nblob, mu, rseg, rblob, repulsive_force_factor, end_force_magnitude,
                           int(wall), max_linear_iter, linear_tol, precision, device)
        cfg = SimConfig(mob, kb, kt, dt, num_euler_steps, max_broyden_iter, tol, jacobian_confidence, body_radius)
        F = nswim * nfil
        self.nswim, self.nfil, self.nseg, self.nblob = nswim, nfil, nseg, nblob
        self.wall = bool(wall)
        self.F, self.S = F, F * nseg
        body_x0 = np.zeros((nswim, 3)) if body_x0 is None else body_x0

        def per_fil(p):
            if p is None:
                return np.zeros((F, 3))
            p = np.asarray(p, dtype=np.float64)
            return np.tile(p.reshape(1, 3), (F, 1)) if p.size == 3 else p.reshape(F, 3)

        blob_refs = np.zeros((0, 3)) if blob_refs is None else blob_refs
        arrays = [_c(blob_refs), _c(fil_refs), _c(body_x0), _c(per_fil(perturbation1)), _c(per_fil(perturbation2))]
        h = ctypes.c_void_p()
        check(self.lib.gmi_sim_create(ctypes.byref(cfg), *[p for _, p in arrays], ctypes.byref(h)))
        self.handle = h
        self.nt = 0
        if beat is not None:  # dict(amplitude, period, phases, end_force_scale)
            self.set_beat(**beat)

    def prepare(self):
        mob = np.zeros(36)
        check(self.lib.gmi_sim_prepare(self.handle, mob.ctypes.data_as(ctypes.c_void_p)))
        return mob.reshape(6, 6, order="F")

    def step(self, nt=None):
        nt = self.nt if nt is None else nt
        b, g = ctypes.c_int(), ctypes.c_int()
        check(self.lib.gmi_sim_step(self.handle, nt, ctypes.byref(b), ctypes.byref(g)))
        self.nt = nt + 1
        return b.value, g.value

    def state(self, name):
        field, cols = STATE[name]
        rows = {"body_x": self.nswim, "body_q": self.nswim, "body_u": self.nswim, "body_v": self.nswim,
                "lam": (self.nseg - 1) * self.F, "tether": self.F, "clamp": self.F,
                "blob_f": self.nswim * self.nblob}.get(name, self.S)
        out = np.zeros((rows, cols))
        check(self.lib.gmi_sim_get_state(self.handle, field, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    # -- checkpoints and time series in the reference's formats ------------
    def export_backup(self) -> np.ndarray:
        n = ctypes.c_longlong()
        check(self.lib.gmi_sim_backup_count(self.handle, ctypes.byref(n)))
        out = np.zeros(n.value)
        check(self.lib.gmi_sim_export_backup(self.handle, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def import_backup(self, values) -> None:
        """Restore a backup; call prepare() again before stepping (the body
        reference matrices follow the restored state)."""
        n = ctypes.c_longlong()
        check(self.lib.gmi_sim_backup_count(self.handle, ctypes.byref(n)))
        v, p = _c(values)
        if v.size != n.value:
            raise ValueError(f"backup holds {v.size} values, this simulation needs {n.value}")
        check(self.lib.gmi_sim_import_backup(self.handle, p))

    def write_backup(self, path, nt_completed, digits=formats.DIGITS):
        formats.write_backup(path, nt_completed, self.export_backup(), digits)

    def read_backup(self, path) -> int:
        """Restore the state of a .backup file; returns its completed-step
        count, the step to continue from."""
        nt, values = formats.read_backup(path)
        self.import_backup(values)
        self.nt = nt
        return nt

    def write_step_data(self, prefix, nt, digits=formats.DIGITS):
        """Append step nt to the reference's .dat files under prefix."""
        formats.write_step_data(prefix, nt, self.state("seg_q"), self.state("body_x"), self.state("body_q"),
                                self.state("seg_v"), self.state("seg_f_internal"),
                                None if self.wall else self.state("body_v"),
                                None if self.wall else self.state("blob_f"), digits)

    def set_beat(self, amplitude, period, phases, end_force_scale=0.0):
        """Prescribed preferred-curvature beat (gmi_sim_set_beat): the
        filaments' preferred bending curvature is amplitude sin(2 pi t /
        period + phase), phases one per filament; end_force_scale 0 turns
        the end force off."""
        ph, p = _c(np.asarray(phases, dtype=np.float64).reshape(-1))
        if ph.size != self.F:
            raise ValueError(f"need {self.F} phases, got {ph.size}")
        check(self.lib.gmi_sim_set_beat(self.handle, float(amplitude), float(period), p, float(end_force_scale)))

    # -- learned initial inverse Jacobian ------------------------------------
    def set_secant_buffer(self, records, capacity=None):
        """Collect one secant-pair record per filament and plain Broyden
        iteration into ``records`` (a float32 CUDA tensor of shape
        (capacity, 24 nseg)); None stops collecting."""
        if records is None:
            check(self.lib.gmi_sim_set_secant_buffer(self.handle, None, 0))
            self._secant = None
            return
        cap = records.shape[0] if capacity is None else capacity
        if records.dtype.itemsize != 4 or records.shape[1] != 24 * self.nseg or not records.is_contiguous():
            raise ValueError("records must be a contiguous float32 tensor of shape (capacity, 24 nseg)")
        self._secant = records
        check(self.lib.gmi_sim_set_secant_buffer(self.handle, ctypes.c_void_p(records.data_ptr()), cap))

    def secant_count(self) -> int:
        n = ctypes.c_longlong()
        check(self.lib.gmi_sim_secant_count(self.handle, ctypes.byref(n)))
        return n.value

    def set_jacobian_probes(self, probes_per_step: int, seed: int = 0, secant_pairs: bool = True):
        """Record ``probes_per_step`` random-direction Jacobian probes per
        iterating step beside (or, with ``secant_pairs=False``, instead of)
        the Broyden iterations' secant pairs (gmi_sim_set_jacobian_probes)."""
        check(self.lib.gmi_sim_set_jacobian_probes(self.handle, probes_per_step, seed, 1 if secant_pairs else 0))

    def set_learned_jacobian(self, net, policy=None):
        """Start Broyden from the network's initial inverse Jacobian
        (``learned.LearnedJacobian``; None: the plain method) under
        ``policy`` (a ``_lib.LearnedPolicy``; None: defaults)."""
        if net is None:
            check(self.lib.gmi_sim_set_learned_jacobian(self.handle, None, 0, None))
            self._net = None
            return
        self._net = net  # keep the network alive while the simulation uses it
        check(self.lib.gmi_sim_set_learned_jacobian(self.handle, net.handle, net.rank,
                                                    ctypes.byref(policy) if policy is not None else None))

    def learned_policy(self):
        out = _lib.LearnedPolicy()
        check(self.lib.gmi_sim_learned_policy(self.handle, ctypes.byref(out)))
        return out

    @property
    def launches(self):
        solver = self.lib.gmi_sim_solver(self.handle)
        return int(self.lib.gmi_context_launch_count(self.lib.gmi_solver_context(solver)))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gmi_sim_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @classmethod
    def from_golden(cls, g, **kw):
        args = dict(wall=bool(g["wall"]) if "wall" in g else False,
                    nswim=int(g["nswim"]) if "nswim" in g else 1,
                    body_x0=g["body_x0"] if "body_x0" in g else None,
                    nfil=int(g["nfil"]), nseg=int(g["nseg"]), nblob=int(g["nblob"]), blob_refs=g["blob_refs"],
                    fil_refs=g["fil_refs"], perturbation1=g["perturbation1"], perturbation2=g["perturbation2"],
                    mu=float(g["mu"]), rseg=float(g["rseg"]), rblob=float(g["rblob"]), kb=float(g["kb"]),
                    kt=float(g["kt"]), dt=float(g["dt"]), end_force_magnitude=float(g["end_force_magnitude"]),
                    repulsive_force_factor=float(g["repulsive_force_factor"]), body_radius=float(g["body_radius"]),
                    tol=float(g["tol"]), linear_tol=float(g["linear_tol"]),
                    max_linear_iter=int(g["max_linear_iter"]))
        args.update(kw)
        return cls(**args)
