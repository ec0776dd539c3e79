"""The allocation-free segment mobility apply, gmi_Mss_mult_noalloc.

It exists for callers that cannot call cudaMalloc (a host program that
owns a fixed device-memory budget, or one that cannot accept the device-wide
synchronisation of cudaMalloc/cudaFree).  Its scratch is a fixed array in
the library instead of memory grown through a gmi_context.  This test calls
it through the C ABI twice in a row, on different inputs, sizes and
precisions, and checks each result against the allocating entry point
gmi_Mss_mult at the tolerances the other pair tests use; it also checks the
size limit.  The file is named so pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

FP64_TOL = 1e-10
FP32C_TOL = 2e-6


def _inputs(n, seed):
    from generic_mobility_interface_class_gb300 import seeding
    x = seeding.random_cube(n, seed=seed)
    f = np.random.default_rng(seed).normal(size=(n, 6))
    return (torch.as_tensor(x, device="cuda"), torch.as_tensor(f, device="cuda"))


def _noalloc(lib, x, f, start, num, precision):
    out = torch.full((num, 6), float("nan"), dtype=torch.float64, device="cuda")
    st = lib.gmi_Mss_mult_noalloc(out.data_ptr(), f.data_ptr(), x.data_ptr(), start, num, x.shape[0], 1.0, 1.0,
                                  precision, None)
    return st, out


def test_noalloc_matches_allocating_entry_point(gmi_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from generic_mobility_interface_class_gb300._lib import check
    from generic_mobility_interface_class_gb300.mobility import Context
    torch.cuda.set_device(0)
    cases = [(4096, 11, 0, 4096, 0, FP64_TOL), (2500, 12, 100, 2000, 1, FP32C_TOL)]
    with Context(0) as ctx:
        for n, seed, start, num, prec, tol in cases:
            x, f = _inputs(n, seed)
            st, got = _noalloc(gmi_lib, x, f, start, num, prec)
            check(st)
            ctx.set_precision(prec)
            want = ctx.mss(x, f, start=start, num=num)
            torch.cuda.synchronize()
            assert rel_err(got.cpu().numpy(), want.cpu().numpy()) < tol


def test_noalloc_rejects_oversize(gmi_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    n = 32769
    x = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    f = torch.zeros((n, 6), dtype=torch.float64, device="cuda")
    st, _ = _noalloc(gmi_lib, x, f, 0, 16, 0)
    assert st == 1  # GMI_ERR_ARG
    assert b"32768" in gmi_lib.gmi_last_error()
