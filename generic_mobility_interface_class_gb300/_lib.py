"""ctypes binding of libgmi.so (include/gmi.h).

The library must have been built (``build.build()``); there is no fallback:
importing a function from a missing library raises GmiLibraryMissing.
"""
from __future__ import annotations

import ctypes
import os
import re
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "_build", "libgmi.so")
HEADER = os.path.join(ROOT, "include", "gmi.h")

GMI_OK = 0
GMI_FP64 = 0
GMI_FP32C = 1
GMI_DF64 = 2  # blob-blob sums only
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
    "gmi_context_set_wait_deadline": ([_P, ctypes.c_longlong], _I),
    "gmi_context_check_bounded_wait": ([_P, _I], _I),
    "gmi_Mss_mult": ([_P, _P, _P, _P, _I, _I, _I, _D, _D], _I),
    "gmi_Mss_mult_wall": ([_P, _P, _P, _P, _I, _I, _I], _I),
    "gmi_Mss_mult_noalloc": ([_P, _P, _P, _I, _I, _I, _D, _D, _I, _P], _I),
    "gmi_Mbb_mult": ([_P, _P, _P, _P, _I, _I, _I, _D, _D], _I),
    "gmi_Msb_mult": ([_P, _P, _P, _P, _P, _I, _I, _I, _I, _D, _D, _D], _I),
    "gmi_Mbs_mult": ([_P, _P, _P, _P, _P, _I, _I, _I, _I, _D, _D, _D], _I),
    "gmi_barrier_forces": ([_P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _I, _D, _D, _D, _I], _I),
    "gmi_autotune": ([_P, _I, _I, _I], _I),
    "gmi_measure_fma_peak": ([_P, _I, ctypes.POINTER(_D)], _I),
    "gmi_tuned_shape": ([_P, _I, _I, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)], _I),
    "gmi_tuned_sources_per_step": ([_P, _I, _I, _I, ctypes.POINTER(_I)], _I),
    "gmi_set_shape": ([_P, _I, _I, _I, _I, _I, _I, _I], _I),
    "gmi_solver_create": ([_P, ctypes.POINTER(_P)], _I),
    "gmi_solver_destroy": ([_P], _I),
    "gmi_solver_host_arrays": ([_P, _P], _I),
    "gmi_solver_context": ([_P], _P),
    "gmi_solver_copy_segment_positions_to_device": ([_P], _I),
    "gmi_solver_copy_segment_forces_to_device": ([_P], _I),
    "gmi_solver_copy_blob_positions_to_device": ([_P], _I),
    "gmi_solver_copy_blob_forces_to_device": ([_P], _I),
    "gmi_solver_copy_interparticle_blob_forces_to_host": ([_P], _I),
    "gmi_solver_copy_blob_velocities_to_host": ([_P], _I),
    "gmi_solver_copy_segment_velocities_to_host": ([_P], _I),
    "gmi_solver_apply_interparticle_forces": ([_P], _I),
    "gmi_solver_wait_for_device": ([_P], _I),
    "gmi_solver_evaluate_segment_segment_mobility": ([_P], _I),
    "gmi_solver_evaluate_segment_blob_mobility": ([_P], _I),
    "gmi_solver_evaluate_blob_blob_mobility": ([_P], _I),
    "gmi_solver_evaluate_blob_segment_mobility": ([_P], _I),
    "gmi_solver_set_blob_references": ([_P, _P], _I),
    "gmi_solver_make_body_reference_matrices": ([_P, _P, _P, _P, _P], _I),
    "gmi_solver_set_body_reference_matrices": ([_P, _P, _P], _I),
    "gmi_solver_compute_velocities": ([_P, _P, _P, _P, ctypes.POINTER(_I)], _I),
    "gmi_solver_compute_velocities_prescribed": ([_P, _P, _P, _P, _P, ctypes.POINTER(_I)], _I),
    "gmi_solver_set_generalised_force_refs": ([_P, _P, _I], _I),
    "gmi_solver_compute_velocities_prescribed_dynamic": ([_P, _P, _P, _P, _P, _P, _P, ctypes.POINTER(_I)], _I),
    "gmi_solver_last_linear_solve": ([_P, ctypes.POINTER(_I), ctypes.POINTER(_D)], _I),
    "gmi_solver_set_strict_convergence": ([_P, _I], _I),
    "gmi_solver_get_v_bodies": ([_P, _P], _I),
    "gmi_solver_set_v_bodies": ([_P, _P], _I),
    "gmi_sim_create": ([_P, _P, _P, _P, _P, _P, ctypes.POINTER(_P)], _I),
    "gmi_sim_destroy": ([_P], _I),
    "gmi_sim_solver": ([_P], _P),
    "gmi_sim_prepare": ([_P, _P], _I),
    "gmi_sim_step": ([_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I)], _I),
    "gmi_sim_get_state": ([_P, _I, _P], _I),
    "gmi_sim_backup_count": ([_P, ctypes.POINTER(ctypes.c_longlong)], _I),
    "gmi_sim_export_backup": ([_P, _P], _I),
    "gmi_sim_import_backup": ([_P, _P], _I),
    "gmi_mlp_create": ([_I, _I, _I, _I, ctypes.c_ulonglong, ctypes.POINTER(_P)], _I),
    "gmi_mlp_destroy": ([_P], _I),
    "gmi_mlp_param_count": ([_P, ctypes.POINTER(ctypes.c_longlong)], _I),
    "gmi_mlp_param_offsets": ([_P, _P], _I),
    "gmi_mlp_get_params": ([_P, _P, ctypes.c_longlong], _I),
    "gmi_mlp_set_params": ([_P, _P, ctypes.c_longlong], _I),
    "gmi_mlp_forward": ([_P, _P, _I, _P], _I),
    "gmi_mlp_backward": ([_P, _P, _I, _P], _I),
    "gmi_mlp_secant_loss": ([_P, _P, ctypes.c_longlong, _I, _I, _P, ctypes.POINTER(_D), _P], _I),
    "gmi_mlp_train_secant": ([_P, _P, ctypes.c_longlong, _I, _I, _I, _I, ctypes.c_float, ctypes.c_ulonglong, _P],
                             _I),
    "gmi_mlp_launch_count": ([_P], ctypes.c_longlong),
    "gmi_learned_policy_init": ([_P], None),
    "gmi_learned_policy_use_learned": ([_P], _I),
    "gmi_learned_policy_iteration_cap": ([_P, _I], _I),
    "gmi_learned_policy_record": ([_P, _I, _I, _I], None),
    "gmi_seed_sphere_repulsive": ([_I, _I, _I, _P, ctypes.POINTER(_I)], _I),
    "gmi_sim_set_beat": ([_P, _D, _D, _P, _D], _I),
    "gmi_sim_set_secant_buffer": ([_P, _P, ctypes.c_longlong], _I),
    "gmi_sim_secant_count": ([_P, ctypes.POINTER(ctypes.c_longlong)], _I),
    "gmi_sim_set_jacobian_probes": ([_P, _I, ctypes.c_ulonglong, _I], _I),
    "gmi_sim_set_learned_jacobian": ([_P, _P, _I, _P], _I),
    "gmi_sim_learned_policy": ([_P, _P], _I),
}


class SolverConfig(ctypes.Structure):
    """gmi_solver_config (include/gmi.h)."""
    _fields_ = [("nswim", _I), ("nfil", _I), ("nseg", _I), ("nblob", _I), ("mu", _D), ("rseg", _D),
                ("rblob", _D), ("repulsive_force_factor", _D), ("end_force_magnitude", _D), ("wall", _I),
                ("max_linear_iter", _I), ("linear_tol", _D), ("precision", _I), ("device", _I)]


class SimConfig(ctypes.Structure):
    """gmi_sim_config (include/gmi.h)."""
    _fields_ = [("mobility", SolverConfig), ("kb", _D), ("kt", _D), ("dt", _D), ("num_euler_steps", _I),
                ("max_broyden_iter", _I), ("tol", _D), ("jacobian_confidence", _D), ("body_radius", _D)]


class LearnedPolicy(ctypes.Structure):
    """gmi_learned_policy (include/gmi.h)."""
    _fields_ = [("calibration_steps", _I), ("window", _I), ("max_regressions", _I), ("margin", _D),
                ("cap_factor", _D), ("mode", _I), ("steps_plain", _I), ("steps_learned", _I), ("regressions", _I),
                ("plain_iters_sum", _D), ("recent", _I * 64), ("recent_count", _I)]


class HostArrays(ctypes.Structure):
    """gmi_host_arrays (include/gmi.h)."""
    _fields_ = [(name, ctypes.POINTER(_D)) for name in
                ("v_segs_host", "v_blobs_host", "x_segs_host", "x_blobs_host", "f_segs_host", "f_blobs_host",
                 "f_blobs_repulsion_host")]

_lib = None
_load_lock = threading.Lock()


def header_symbols() -> list[str]:
    """Names of the functions include/gmi.h declares."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"GMI_API\s+[\w\s\*]*?\b(gmi_\w+)\s*\(", text)))


def load() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    with _load_lock:  # the swimmers of a batch are built on several threads
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
