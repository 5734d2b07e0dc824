"""The C ABI library on a machine without a GPU: it loads, exports every
function that include/maxwell_gb300.h declares, and reports the missing
device instead of computing anything."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import maxwell_gb300 as mx


@pytest.fixture(scope="module")
def built():
    from maxwell_gb300.build import build
    return build()


def test_library_exports_every_declared_function(built):
    names = mx.header_functions()
    assert len(names) > 50
    lib = C.CDLL(built)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_exports_are_c_linkage(built):
    out = subprocess.run(["nm", "-D", "--defined-only", built], capture_output=True, text=True).stdout
    syms = {line.split()[-1] for line in out.splitlines() if line.strip()}
    for n in mx.header_functions():
        assert n in syms, n


def test_no_device_means_errors_not_results(built):
    if mx.lib().mxg_device_ok():
        pytest.skip("a GPU is present")
    g = mx.lib().new_grid2d_gpu(8, 8, 0.125, 0.125, 1)
    assert not g   # allocation on a missing device fails loudly
    o = mx.SolveOpts(8, 1, 4, 6, 1, 1, 5, 5, 2, 5, 2, 1, 1, 1, 1, 1e-8)
    s = mx.lib().mxg_solver_new(C.byref(o), np.ones(256).ctypes.data_as(C.c_void_p))
    assert not s


def test_solver_rejects_bad_options(built):
    bad = [mx.SolveOpts(7, 1, 4, 6, 1, 1, 5, 5, 2, 5, 2, 1, 1, 1, 1, 1e-8),    # odd n0
           mx.SolveOpts(8, 1, 8, 6, 1, 1, 5, 5, 2, 5, 2, 1, 1, 1, 1, 1e-8),    # ieigs > m
           mx.SolveOpts(8, 1, 4, 40, 1, 1, 5, 5, 2, 5, 2, 1, 1, 1, 1, 1e-8),   # m > 16
           mx.SolveOpts(8, 1, 4, 6, 1, 1, 5, 5, 2, 5, 2, 1, 1, 0, 1, 1e-8),    # wave 0
           mx.SolveOpts(8, 1, 4, 6, 1, 1, 5, 5, 2, 5, 2, 1, 1, 1, 1, 1e-8, 2)]  # no such smoother
    for o in bad:
        assert not mx.lib().mxg_solver_new(C.byref(o), np.ones(256).ctypes.data_as(C.c_void_p))


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    monkeypatch.setattr(mx, "_lib", None)
    monkeypatch.setattr(mx, "LIB_PATH", str(tmp_path / "absent.so"))
    with pytest.raises(ImportError):
        mx.lib()
