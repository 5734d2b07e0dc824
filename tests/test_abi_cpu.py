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
    assert mx.lib().mxg_set_device(0) != 0   # no device to select


def test_solver_rejects_bad_options(built):
    bad = [mx.SolveOpts(7, 1, 4, 6, 1, 1, 5, 5, 2, 5, 2, 1, 1, 1, 1, 1e-8),    # odd n0
           mx.SolveOpts(8, 1, 8, 6, 1, 1, 5, 5, 2, 5, 2, 1, 1, 1, 1, 1e-8),    # ieigs > m
           mx.SolveOpts(8, 1, 4, 40, 1, 1, 5, 5, 2, 5, 2, 1, 1, 1, 1, 1e-8),   # m > 32
           mx.SolveOpts(8, 1, 4, 6, 1, 1, 5, 5, 2, 5, 2, 1, 1, 0, 1, 1e-8),    # wave 0
           mx.SolveOpts(8, 1, 4, 6, 1, 1, 5, 5, 2, 5, 2, 1, 1, 1, 1, 1e-8, 2),  # no such smoother
           mx.SolveOpts(8, 1, 4, 6, 1, 1, 5, 5, 2, 5, 2, 1, 1, 1, 1, 1e-8, 1, 0.0, ord("3"))]  # extrapolation
    for o in bad:
        assert not mx.lib().mxg_solver_new(C.byref(o), np.ones(256).ctypes.data_as(C.c_void_p))


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    monkeypatch.setattr(mx, "_lib", None)
    monkeypatch.setattr(mx, "LIB_PATH", str(tmp_path / "absent.so"))
    with pytest.raises(ImportError):
        mx.lib()


@pytest.mark.parametrize("cc, lang, std", [("gcc", "c", "c99"), ("gcc", "c", "c11"), ("g++", "c++", "c++17")])
def test_header_compiles_for_c_and_cpp_callers(cc, lang, std):
    """The boundary header is plain C that a reference caller (C99, OpenMP)
    or a C++ host includes without warnings."""
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    src = '#include "maxwell_gb300.h"\nint main(void) { return 0; }\n'
    r = subprocess.run([cc, "-x", lang, f"-std={std}", "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only",
                        "-I", inc, "-"], input=src, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_c_caller_links_every_declared_function(built):
    """A C program that takes the address of every declared function links
    against the library: declarations and exports agree in name and
    linkage (nothing runs)."""
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    names = mx.header_functions()
    body = "\n".join(f"  (void) &{n};" for n in names)
    src = f'#include "maxwell_gb300.h"\nint main(void) {{\n{body}\n  return 0;\n}}\n'
    r = subprocess.run(["gcc", "-x", "c", "-std=c11", "-I", inc, "-", "-o", os.devnull, "-L", os.path.dirname(built),
                        "-l:" + os.path.basename(built)], input=src, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_c_caller_example_compiles(built):
    """tests/c_caller_example.c, a reference-style C caller of the solver,
    compiles against the header without warnings and links against the
    library."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = os.path.join(root, "tests", "c_caller_example.c")
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-c", src, "-o", os.devnull,
                        "-I", os.path.join(root, "include")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_protocol_file_matches_the_reference_format(built, golden, tmp_path):
    """mxg_write_protocol writes the header of the reference driver's
    protocol file line for line (the header its own run wrote, kept in the
    driver-curve fixture) and the per-point lines in its format: the values
    read back as the driver's protocol is read.  Host code only."""
    g = golden("bloch_curve_n16_kivshar.npz")
    lam, chern = g["lam"], g["chern"]
    nk, m = lam.shape
    f = tmp_path / "bloch2d.dat"
    mx.write_protocol(str(f), "Kivshar", int(g["n0"]), int(g["L"]), lam, steps=g["iterations"],
                      seconds=np.full(nk, 0.25), chern=chern, sign=np.zeros(nk, np.int32),
                      extrapolation="2", stopping="r", continuity="s")
    lines = f.read_text().splitlines()
    header = [ln for ln in lines if ln.startswith("#")]
    assert header == list(g["protocol_header"])
    rows = [ln.split() for ln in lines if not ln.startswith("#")]
    assert len(rows) == nk and len(rows[0]) == 1 + m
    for l, v in enumerate(rows):
        assert int(v[0]) == l
        assert np.allclose([float(x) for x in v[1:1 + m]], lam[l], atol=5e-7)
        if l:
            assert int(v[1 + m]) == int(g["iterations"][l])
            assert float(v[3 + m]) == pytest.approx(0.25 * l, abs=0.06)   # printed with one decimal
            c = [float(x) for x in v[4 + m:4 + m + 2 * chern.shape[1]]]
            assert np.allclose(c[0::2], chern[l].real, atol=5e-7) and np.allclose(c[1::2], chern[l].imag, atol=5e-7)
            assert int(v[-1]) == 0


def test_tuning_get_set_without_gpu(built):
    """The launch-shape tunables are host state: get/set work without a GPU,
    out-of-range shapes are refused, the autotuner needs a device."""
    import maxwell_gb300 as mx
    t0 = mx.get_tuning()
    assert t0 == {"gram_waves": 4, "combine_ctas": 2, "residual_sites": 32, "node_strip": 0, "node_band": 16,
                  "restrict_strip_log2": 25}
    mx.set_tuning(8, 1, 64, 64, 8, 0)
    want = {"gram_waves": 8, "combine_ctas": 1, "residual_sites": 64, "node_strip": 64, "node_band": 8,
            "restrict_strip_log2": 0}
    assert mx.get_tuning() == want
    for bad in ((0, 2, 32), (4, 17, 32), (4, 2, 0), (65, 2, 32), (4, 2, 32, 96, 8), (4, 2, 32, 64, 0),
                (4, 2, 32, 0, 16, -1), (4, 2, 32, 0, 16, 63)):
        with pytest.raises(RuntimeError):
            mx.set_tuning(*bad)
    assert mx.get_tuning() == want
    mx.set_tuning(**t0)
    with pytest.raises(RuntimeError):
        mx.autotune(64, 2, 4)
