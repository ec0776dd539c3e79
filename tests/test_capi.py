"""The C-ABI library loads, exports exactly what include/gmi.h declares, and
fails with a status code (never a crash) where it cannot run."""
import ctypes
import os
import subprocess

import pytest


def test_header_symbols_exported(gmi_lib):
    from generic_mobility_interface_class_gb300 import _lib
    declared = _lib.header_symbols()
    assert len(declared) >= 15
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    extra = sorted(s for s in exported if s.startswith("gmi_") and s not in declared)
    assert not extra, f"exported but not declared: {extra}"


def test_python_signatures_cover_header(gmi_lib):
    from generic_mobility_interface_class_gb300 import _lib
    assert set(_lib.header_symbols()) == set(_lib.SIGNATURES)


def test_version_and_error_string(gmi_lib):
    assert gmi_lib.gmi_version() >= 100
    assert isinstance(gmi_lib.gmi_last_error(), bytes)


def test_null_arguments_rejected(gmi_lib):
    """Argument checks run before any CUDA call, so they work without a GPU."""
    from generic_mobility_interface_class_gb300._lib import check, GmiError
    with pytest.raises(GmiError) as e:
        check(gmi_lib.gmi_context_create(0, None))
    assert e.value.status == 1
    with pytest.raises(GmiError) as e:
        check(gmi_lib.gmi_Mss_mult(None, None, None, None, 0, 1, 1, 1.0, 1.0))
    assert e.value.status == 1
    assert gmi_lib.gmi_context_set_precision(None, 0) == 1


def test_context_create_without_gpu_returns_status(gmi_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    st = gmi_lib.gmi_context_create(0, ctypes.byref(h))
    assert st in (1, 2)  # GMI_ERR_ARG (no such device) or GMI_ERR_CUDA
    assert not h.value


def test_library_missing_is_loud(tmp_path, monkeypatch):
    from generic_mobility_interface_class_gb300 import _lib
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(_lib.GmiLibraryMissing):
        _lib.load()


def test_reference_side_adapter_compiles(gmi_lib):
    """The reference-side binding (adapter/gb300_mobility_solver.cpp) compiles
    against the reference's own headers (config.hpp, mobility_solver.hpp,
    swimmer.hpp); skipped where the reference tree is absent."""
    from oracle import reference_dir
    ref = reference_dir()
    if not os.path.isfile(os.path.join(ref, "mobility_solver.hpp")):
        pytest.skip("reference tree not present")
    from generic_mobility_interface_class_gb300 import _lib
    adapter = os.path.join(_lib.PKG, "adapter")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I" + ref, "-I" + os.path.join(_lib.ROOT, "include"),
                        "-I" + adapter, os.path.join(adapter, "gb300_mobility_solver.cpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_reference_side_adapter_compiles_for_prescribed_cilia(gmi_lib, tmp_path):
    """The adapter's prescribed-cilia branch (CILIA_TYPE 3, with and without
    DYNAMIC_PHASE_EVOLUTION) compiles against the reference's headers, with the
    reference's config.hpp set for it; skipped where the reference tree is
    absent."""
    from oracle import reference_dir
    ref = reference_dir()
    if not os.path.isfile(os.path.join(ref, "mobility_solver.hpp")):
        pytest.skip("reference tree not present")
    from generic_mobility_interface_class_gb300 import _lib
    from oracle.ref_solver import build_ref_solver as brs
    adapter = os.path.join(_lib.PKG, "adapter")
    for dyn in ("true", "false"):
        spec = dict(brs.COMMON)
        spec.update(CILIA_TYPE="3", DYNAMIC_PHASE_EVOLUTION=dyn)
        cfg = tmp_path / dyn
        cfg.mkdir()
        (cfg / "config.hpp").write_text(brs.config_text(spec))
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I" + str(cfg), "-I" + ref,
                            "-I" + os.path.join(_lib.ROOT, "include"), "-I" + adapter, "-include",
                            str(cfg / "config.hpp"), os.path.join(adapter, "gb300_mobility_solver.cpp")],
                           capture_output=True, text=True)
        assert r.returncode == 0, (dyn, r.stderr[-3000:])
