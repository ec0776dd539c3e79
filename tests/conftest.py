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
    got = np.asarray(got)
    want = np.asarray(want)
    scale = np.max(np.abs(want))
    return float(np.max(np.abs(got - want)) / (scale if scale > 0 else 1.0))


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
