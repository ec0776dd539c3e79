import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libgmi.so")


def golden_cases(prefix="pairs_"):
    return sorted(os.path.basename(p)[len(prefix):-4] for p in glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def load_golden(name, prefix="pairs_"):
    d = np.load(os.path.join(GOLDEN, f"{prefix}{name}.npz"))
    return {k: d[k] for k in d.files}


def rel_err(got, want):
    """max |got - want| / max |want|: the error normalised by the largest
    value of the whole output."""
    got = np.asarray(got)
    want = np.asarray(want)
    scale = np.max(np.abs(want))
    return float(np.max(np.abs(got - want)) / (scale if scale > 0 else 1.0))


def per_target_rel(got, want):
    """Per-target relative error of velocity outputs: for every target and
    every 3-vector block of its row (v, and omega for 6-column rows),
    |got - want| / |want|.  Returns (max, rms) over all blocks.  Unlike
    rel_err, a target with a small velocity is held to its own magnitude."""
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    assert got.shape == want.shape and got.shape[-1] % 3 == 0
    g = got.reshape(-1, 3)
    w = want.reshape(-1, 3)
    den = np.linalg.norm(w, axis=1)
    assert np.all(den > 0), "per-target error needs non-zero reference rows"
    r = np.linalg.norm(g - w, axis=1) / den
    return float(r.max()), float(np.sqrt(np.mean(r * r)))


@pytest.fixture(scope="session")
def oracle_built():
    from oracle import rpy
    rpy.build()
    return rpy


@pytest.fixture(scope="session")
def gmi_lib():
    from generic_mobility_interface_class_gb300 import build
    build.build()
    from generic_mobility_interface_class_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def gpu_ctx(gmi_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from generic_mobility_interface_class_gb300.mobility import Context
    ctx = Context(0)
    yield ctx
    ctx.close()
