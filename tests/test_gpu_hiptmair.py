"""The Hiptmair cycle and its point smoother (hcycle_edge2d,
gs*_simple_edge2d) through the C ABI against the reference's own golden
vectors (tests/golden/hiptmair_n16.npz), the solver preconditioned by the
Hiptmair cycle against the reference's eigenvalues, and the contraction
rates of the two cycles on a constant-coefficient problem.  Tolerances:
complex128 1e-11 relative (1e-10 for whole cycles), complex64 1e-4."""
import ctypes as C

import numpy as np
import pytest

import maxwell_gb300 as mx

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def arr(objs):
    return C.cast((C.c_void_p * len(objs))(*[o.h for o in objs]), C.c_void_p)


@pytest.mark.parametrize("prec", [mx.C128, mx.C64])
@pytest.mark.parametrize("direction", [0, 1, 2])
def test_point_smoother_matches_reference(golden, prec, direction):
    g0 = golden("hiptmair_n16.npz")
    n = int(g0["n0"]) << int(g0["L"])
    g = mx.Grid(n, 1, g0["kappa"], [[complex(g0["xf"]), complex(g0["yf"])]])
    eb, ex = mx.Edge(g, 1, prec, g0["b"]), mx.Edge(g, 1, prec, g0["x"])
    fn = [mx.lib().gsforward_simple_edge2d_gpu, mx.lib().gsbackward_simple_edge2d_gpu,
          mx.lib().gssymm_simple_edge2d_gpu][direction]
    mx.check(fn(mx.fz(1.0), mx.fz(1.0), eb.h, ex.h))
    want = g0["simple_" + ["fwd", "bwd", "symm"][direction]]
    assert rel(ex.get()[0, 0], want) < (1e-11 if prec == mx.C128 else 1e-4)


def hierarchy(g0, m=1, prec=mx.C128):
    n0, L = int(g0["n0"]), int(g0["L"])
    grids = [mx.Grid(n0 << L, 1, g0["kappa"], [[complex(g0["xf"]), complex(g0["yf"])]])]
    for _ in range(L):
        grids.append(grids[-1].coarsen())
    grids = grids[::-1]
    mk = lambda cls: [cls(gr, m, prec) for gr in grids]
    return grids, mk(mx.Edge), mk(mx.Edge), mk(mx.Edge), mk(mx.Node), mk(mx.Node)


def test_hcycle_matches_reference(golden):
    g0 = golden("hiptmair_n16.npz")
    n0, L = int(g0["n0"]), int(g0["L"])
    for key, coarse, cycles in (("hcycle", True, 2), ("hcycle_nocoarse", False, 1)):
        grids, b, x, d, bg, xg = hierarchy(g0)
        b[L].put(g0["b"])
        Ac = None
        if coarse:
            Ac = mx.Matrix(2 * n0 * n0, 1)
            info = np.zeros(1, np.int32)
            mx.check(mx.lib().densematrix_edge2d_gpu(mx.fz(1.0), mx.fz(1.0), grids[0].h, Ac.h))
            mx.check(mx.lib().potrf_matrix_gpu(Ac.h, mx._ptr(info)))
        for _ in range(cycles):
            mx.check(mx.lib().hcycle_edge2d_gpu(L, 2, Ac.h if Ac else None, arr(b), arr(x), arr(d), arr(bg),
                                                arr(xg)))
        assert rel(x[L].get()[0, 0], g0[key]) < 1e-10, key


@pytest.mark.parametrize("precision", [0, 1])
def test_solver_with_hiptmair_cycle(golden, precision):
    """The block solver with the Hiptmair cycle as its preconditioner
    (mxg_solve_opts.smoother = 2) converges to the reference's eigenvalues."""
    g = golden("eigs_n32_disc.npz")
    ie, m = int(g["ieigs"]), int(g["m"])
    s = mx.Solver(g["kappa"], n0=int(g["n0"]), L=int(g["L"]), ieigs=ie, m=m, method=1, precision=precision,
                  max_nested=40, max_steps=60, wave=len(g["factors"]), relative=0, tol=float(g["tol"]), smoother=2)
    lam, steps, res = s.solve(g["factors"])
    assert res[:, :ie].max() <= float(g["tol"])
    assert (np.abs(lam[:, :ie] - g["lam"][:, :ie]) / g["lam"][:, :ie]).max() < 1e-8


def test_cycle_rates():
    """Contraction of the reference-order AFW V-cycle and of the Hiptmair
    cycle on a constant-coefficient 64^2 problem (2 smoothing steps, coarse
    dense solve on 8^2): both contract, at rates near the reference's own
    measurements at 512^2 (AFW 0.45, Hiptmair 0.47-0.50)."""
    n0, L = 8, 3
    rates = {}
    rng = np.random.default_rng(4)
    for cycle in ("vcycle", "hcycle"):
        fine = mx.Grid(n0 << L, 1, None, [[np.exp(0.3j), np.exp(1.1j)]])
        grids = [fine]
        for _ in range(L):
            grids.append(grids[-1].coarsen())
        grids = grids[::-1]
        mk = lambda cls: [cls(gr, 1, mx.C128) for gr in grids]
        b, x, d, bg, xg = mk(mx.Edge), mk(mx.Edge), mk(mx.Edge), mk(mx.Node), mk(mx.Node)
        Ac = mx.Matrix(2 * n0 * n0, 1)
        info = np.zeros(1, np.int32)
        mx.check(mx.lib().densematrix_edge2d_gpu(mx.fz(1.0), mx.fz(1.0), grids[0].h, Ac.h))
        mx.check(mx.lib().potrf_matrix_gpu(Ac.h, mx._ptr(info)))
        nn = 2 * (n0 << L) ** 2
        x[L].put(rng.standard_normal(nn) + 1j * rng.standard_normal(nn))     # b = 0: x is the error
        norms = [np.linalg.norm(x[L].get())]
        for _ in range(6):
            if cycle == "vcycle":
                mx.check(mx.lib().vcycle_edge2d_gpu(L, 2, Ac.h, arr(b), arr(x), arr(d)))
            else:
                mx.check(mx.lib().hcycle_edge2d_gpu(L, 2, Ac.h, arr(b), arr(x), arr(d), arr(bg), arr(xg)))
            norms.append(np.linalg.norm(x[L].get()))
        rates[cycle] = norms[-1] / norms[-2]
    assert rates["vcycle"] < 0.6 and rates["hcycle"] < 0.6, rates
