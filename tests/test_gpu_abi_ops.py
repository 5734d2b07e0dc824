"""The rest of the reference's edge2d / node2d / grid2d / linalg interface
through the C ABI: vector operations, null-space products, the block Gram
and combination, M-orthonormalisation, one PINVIT step, the permittivity
pattern and the coarse solve, each against the oracle restatement or the
reference's own golden vectors, batched over k-points and vectors.

Tolerances: FP64 and float-float storage 1e-12 relative, FP32 storage 2e-5;
exact equality for copies, swaps and the permittivity pattern."""
import ctypes as C

import numpy as np
import pytest

import maxwell_gb300 as mx

pytestmark = pytest.mark.gpu

TOL = {mx.C128: 1e-12, mx.CDD: 1e-12, mx.C64: 2e-5}
FACTORS = np.array([[np.exp(0.7j), np.exp(-1.3j)], [1.0, 1.0], [np.exp(2.9j), np.exp(0.4j)]])


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def cv(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.fixture(scope="module")
def setup():
    rng = np.random.default_rng(23)
    n, K, m = 16, 3, 3
    kap = 1.0 / (1.0 + 11.0 * rng.random(n * n))
    return rng, n, K, m, kap


@pytest.mark.parametrize("prec", [mx.C128, mx.CDD, mx.C64])
def test_edge_vector_ops(oracle, setup, prec):
    rng, n, K, m, kap = setup
    g = mx.Grid(n, K, kap, FACTORS)
    x, y = cv(rng, K, m, 2 * n * n), cv(rng, K, m, 2 * n * n)
    ex, ey = mx.Edge(g, m, prec, x), mx.Edge(g, m, prec, y)
    xs, ys = ex.get(), ey.get()               # as stored (rounded to the precision)
    # scale_edge2d
    mx.check(mx.lib().scale_edge2d_gpu(mx.fz(0.3 - 1.1j), ex.h))
    assert rel(ex.get(), (0.3 - 1.1j) * xs) < TOL[prec]
    ex.put(x)
    # swap_edge2d: contents change hands exactly
    mx.check(mx.lib().swap_edge2d_gpu(ex.h, ey.h))
    assert np.array_equal(ex.get(), ys) and np.array_equal(ey.get(), xs)
    mx.check(mx.lib().swap_edge2d_gpu(ex.h, ey.h))
    # normmax_edge2d, dotprod_edge2d
    out = np.zeros(K * m)
    mx.check(mx.lib().normmax_edge2d_gpu(ex.h, mx._ptr(out)))
    want = np.array([[oracle.normmax(xs[k, v]) for v in range(m)] for k in range(K)]).reshape(-1)
    assert rel(out, want) < 1e-15
    dots = np.zeros(K * m, np.complex128)
    mx.check(mx.lib().dotprod_edge2d_gpu(ex.h, ey.h, mx._ptr(dots)))
    want = np.array([[oracle.dot(xs[k, v], ys[k, v]) for v in range(m)] for k in range(K)]).reshape(-1)
    assert rel(dots, want) < (1e-12 if prec != mx.C64 else 1e-5)
    # nullprod_edge2d, nulladd_edge2d
    xp, yp = np.zeros(K * m, np.complex128), np.zeros(K * m, np.complex128)
    mx.check(mx.lib().nullprod_edge2d_gpu(ex.h, mx._ptr(xp), mx._ptr(yp)))
    want = np.array([[oracle.nullprod_edge(n, xs[k, v]) for v in range(m)] for k in range(K)]).reshape(-1, 2)
    assert rel(xp, want[:, 0]) < 1e-12 and rel(yp, want[:, 1]) < 1e-12
    xa, ya = cv(rng, K * m), cv(rng, K * m)
    mx.check(mx.lib().nulladd_edge2d_gpu(mx._ptr(xa), mx._ptr(ya), ex.h))
    want = np.array([[oracle.nulladd_edge(n, xa[k * m + v], ya[k * m + v], xs[k, v]) for v in range(m)]
                     for k in range(K)])
    assert rel(ex.get(), want) < TOL[prec]


def test_random_edge_and_node():
    """random_edge2d / random_node2d: entries in [-1, 1) + i[-1, 1), the
    same for the same seed, different for another seed, mean near zero."""
    n, K, m = 32, 2, 4
    g = mx.Grid(n, K)
    a, b = mx.Edge(g, m, mx.C128), mx.Edge(g, m, mx.C128)
    mx.check(mx.lib().random_edge2d_gpu(a.h, 12345))
    mx.check(mx.lib().random_edge2d_gpu(b.h, 12345))
    va, vb = a.get(), b.get()
    assert np.array_equal(va, vb)
    assert np.abs(va.real).max() <= 1.0 and np.abs(va.imag).max() <= 1.0
    assert abs(va.real.mean()) < 0.02 and abs(va.imag.mean()) < 0.02
    assert abs(np.var(va.real) - 1.0 / 3.0) < 0.02
    mx.check(mx.lib().random_edge2d_gpu(b.h, 12346))
    assert np.abs(b.get() - va).min() > 0.0 or not np.array_equal(b.get(), va)
    nd = mx.Node(g, m, mx.C64)
    mx.check(mx.lib().random_node2d_gpu(nd.h, 7))
    vn = nd.get()
    assert np.abs(vn.real).max() <= 1.0 and abs(vn.imag.mean()) < 0.03


@pytest.mark.parametrize("prec", [mx.C128, mx.C64])
def test_node_vector_ops(oracle, setup, prec):
    rng, n, K, m, kap = setup
    g = mx.Grid(n, K, kap, FACTORS)
    x, y = cv(rng, K, m, n * n), cv(rng, K, m, n * n)
    nx_, ny_ = mx.Node(g, m, prec, x), mx.Node(g, m, prec, y)
    xs, ys = nx_.get(), ny_.get()
    nz = mx.Node(g, m, mx.C128)
    mx.check(mx.lib().copy_node2d_gpu(nx_.h, nz.h))
    assert np.array_equal(nz.get(), xs)
    mx.check(mx.lib().add_node2d_gpu(mx.fz(0.5 + 2j), ny_.h, nx_.h))
    assert rel(nx_.get(), xs + (0.5 + 2j) * ys) < TOL[prec]
    nx_.put(x)
    mx.check(mx.lib().scale_node2d_gpu(mx.fz(-1.5j), nx_.h))
    assert rel(nx_.get(), -1.5j * xs) < TOL[prec]
    nx_.put(x)
    out = np.zeros(K * m)
    mx.check(mx.lib().norm2_node2d_gpu(nx_.h, mx._ptr(out)))
    want = np.array([[oracle.norm2(xs[k, v]) for v in range(m)] for k in range(K)]).reshape(-1)
    assert rel(out, want) < (1e-13 if prec != mx.C64 else 1e-6)
    mx.check(mx.lib().normmax_node2d_gpu(nx_.h, mx._ptr(out)))
    want = np.array([[oracle.normmax(xs[k, v]) for v in range(m)] for k in range(K)]).reshape(-1)
    assert rel(out, want) < 1e-15
    dots = np.zeros(K * m, np.complex128)
    mx.check(mx.lib().dotprod_node2d_gpu(nx_.h, ny_.h, mx._ptr(dots)))
    want = np.array([[oracle.dot(xs[k, v], ys[k, v]) for v in range(m)] for k in range(K)]).reshape(-1)
    assert rel(dots, want) < (1e-12 if prec != mx.C64 else 1e-5)
    mx.check(mx.lib().center_node2d_gpu(nx_.h))
    want = np.array([[oracle.center_node(n, xs[k, v]) for v in range(m)] for k in range(K)])
    assert rel(nx_.get(), want) < (1e-13 if prec != mx.C64 else 1e-5)


@pytest.mark.parametrize("prec", [mx.C128, mx.CDD])
def test_gram_and_lincomb(oracle, setup, prec):
    """gram_edge2d_gpu (the Ritz products of exp_bloch2d.c:991-996) and
    lincomb_edge2d_gpu (the combination of exp_bloch2d.c:1006-1010)."""
    rng, n, K, _, kap = setup
    m = 5
    g = mx.Grid(n, K, kap, FACTORS)
    x = cv(rng, K, m, 2 * n * n)
    ex = mx.Edge(g, m, prec, x)
    A = np.zeros((K, m, m), np.complex128)
    M = np.zeros((K, m, m), np.complex128)
    mx.check(mx.lib().gram_edge2d_gpu(ex.h, mx._ptr(A), mx._ptr(M)))
    A, M = A.transpose(0, 2, 1), M.transpose(0, 2, 1)   # column-major per k
    for k in range(K):
        for i in range(m):
            for j in range(m):
                # entry (i, j) = u_i^H K u_j = energyprod_edge2d(u_i, u_j), which
                # returns CONJ(sum conj(u_j) (K u_i)) (edge2d.c:1958)
                wa = oracle.energyprod_edge(n, kap, *FACTORS[k], 1.0, 1.0, x[k, i], x[k, j])
                wm = oracle.massprod_edge(n, *FACTORS[k], x[k, i], x[k, j])
                assert abs(A[k, i, j] - wa) < 1e-11 * abs(A[k]).max()
                assert abs(M[k, i, j] - wm) < 1e-11 * abs(M[k]).max()
    coef = cv(rng, K, m, m)                      # coef[k][i][j]
    ey = mx.Edge(g, m, prec)
    cm = np.ascontiguousarray(coef.transpose(0, 2, 1))   # column-major
    mx.check(mx.lib().lincomb_edge2d_gpu(mx._ptr(cm), ex.h, ey.h))
    want = np.einsum("kij,kie->kje", coef, x)
    assert rel(ey.get(), want) < 1e-12


@pytest.mark.parametrize("prec", [mx.C128, mx.CDD])
def test_orthonormalize(oracle, setup, prec):
    """orthonormalize_edge2d_gpu: the result is M-orthonormal and spans the
    same nested subspaces (R = Q^H M X upper triangular with a positive
    real diagonal reproduces X)."""
    rng, n, K, _, kap = setup
    m = 6
    g = mx.Grid(n, K, kap, FACTORS)
    x = cv(rng, K, m, 2 * n * n)
    ex = mx.Edge(g, m, prec, x)
    info = np.zeros(K, np.int32)
    mx.check(mx.lib().orthonormalize_edge2d_gpu(ex.h, mx._ptr(info)))
    assert not info.any()
    q = ex.get()
    for k in range(K):
        # massprod_edge(a, b) = a^H M b
        G = np.array([[oracle.massprod_edge(n, *FACTORS[k], q[k, i], q[k, j]) for j in range(m)] for i in range(m)])
        assert np.abs(G - np.eye(m)).max() < 1e-11
        R = np.array([[oracle.massprod_edge(n, *FACTORS[k], q[k, i], x[k, j]) for j in range(m)] for i in range(m)])
        assert np.abs(np.tril(R, -1)).max() < 1e-11 * np.abs(R).max()
        assert (np.diag(R).real > 0).all() and np.abs(np.diag(R).imag).max() < 1e-11 * np.abs(R).max()
        assert rel(np.einsum("ij,ie->je", R, q[k]), x[k]) < 1e-12
    # a dependent column: column 3 repeats column 1
    x2 = x.copy()
    x2[:, 3] = x2[:, 1]
    e2 = mx.Edge(g, m, prec, x2)
    assert mx.lib().orthonormalize_edge2d_gpu(e2.h, mx._ptr(info)) == -3     # MXG_ECONV
    assert (info == 4).all()
    assert np.array_equal(e2.get(), mx.Edge(g, m, prec, x2).get())          # left unchanged


def test_pinvit_step_matches_reference(golden):
    """pinvit_edge2d_gpu against the reference's pinvit_edge2d
    (edge2d.c:6298-6328, golden vector of its own build): 2 V-cycles with 2
    smoothing steps, 5 node V-cycles of lifting, lambda = 40."""
    g0 = golden("vcycle_n16.npz")
    n0, L, xf, yf = int(g0["n0"]), int(g0["L"]), complex(g0["xf"]), complex(g0["yf"])
    grids = [mx.Grid(n0 << L, 1, g0["kappa"], [[xf, yf]])]
    for _ in range(L):
        grids.append(grids[-1].coarsen())
    grids = grids[::-1]
    mk = lambda cls: [cls(gr, 1, mx.C128) for gr in grids]
    b, x, d = mk(mx.Edge), mk(mx.Edge), mk(mx.Edge)
    bg, xg, dg = mk(mx.Node), mk(mx.Node), mk(mx.Node)
    Ae, An = mx.Matrix(2 * n0 * n0, 1), mx.Matrix(n0 * n0, 1)
    info = np.zeros(1, np.int32)
    mx.check(mx.lib().densematrix_edge2d_gpu(mx.fz(1.0), mx.fz(1.0), grids[0].h, Ae.h))
    mx.check(mx.lib().potrf_matrix_gpu(Ae.h, mx._ptr(info)))
    mx.check(mx.lib().densematrix_node2d_gpu(1, grids[0].h, An.h))
    mx.check(mx.lib().potrf_matrix_gpu(An.h, mx._ptr(info)))
    e = mx.Edge(grids[L], 1, mx.C128, g0["e"])
    arr = lambda objs: C.cast((C.c_void_p * len(objs))(*[o.h for o in objs]), C.c_void_p)
    lam = np.array([40.0])
    mx.check(mx.lib().pinvit_edge2d_gpu(L, 2, 2, 5, mx._ptr(lam), e.h, Ae.h, arr(b), arr(x), arr(d), An.h,
                                        arr(bg), arr(xg), arr(dg)))
    assert rel(e.get()[0, 0], g0["pinvit"]) < 1e-10


def test_potrsv_matches_oracle(oracle, setup):
    """potrsv_matrix_gpu after potrf_matrix_gpu on the coarse edge and node
    matrices of three k-points against the oracle's Cholesky solve."""
    rng, _, K, _, _ = setup
    n = 4
    kap = 1.0 / (1.0 + 11.0 * rng.random(n * n))
    g = mx.Grid(n, K, kap, FACTORS)
    for rows, make in ((2 * n * n, lambda a: mx.lib().densematrix_edge2d_gpu(mx.fz(1.0), mx.fz(1.0), g.h, a)),
                       (n * n, lambda a: mx.lib().densematrix_node2d_gpu(1, g.h, a))):
        A = mx.Matrix(rows, K)
        mx.check(make(A.h))
        dense = A.get()
        info = np.zeros(K, np.int32)
        mx.check(mx.lib().potrf_matrix_gpu(A.h, mx._ptr(info)))
        assert not info.any()
        bvec = cv(rng, K, rows)
        sol = np.ascontiguousarray(bvec.copy())
        mx.check(mx.lib().potrsv_matrix_gpu(A.h, mx._ptr(sol)))
        for k in range(K):
            st, want = oracle.chol_solve(dense[k], bvec[k])
            assert st == 0
            assert rel(sol[k], want) < 1e-11


def test_setpattern_matches_oracle(oracle):
    """setpattern_grid2d_gpu (rasterised on the device) equals the oracle's
    restatement of setpattern_grid2d bit for bit: the config-2 disc, the
    four discs of the surface configuration, and rectangles under circles."""
    cases = [
        (512, [], [[12.0, 0.5, 0.5, 0.3]], 1.0),
        (256, [], [[10.0, cx, cy, 0.15] for cy in (0.25, 0.75) for cx in (0.25, 0.75)], 1.0),
        (64, [[4.0, 0.1, 0.2, 0.5, 0.25], [8.9, 0.0, 0.0, 0.25, 1.0]], [[12.0, 0.6, 0.6, 0.2]], 2.0),
    ]
    for n, rects, circles, base in cases:
        g = mx.Grid(n, 1)
        g.set_pattern(rects, circles, base)
        want = oracle.pattern_kappa(n, rects, circles, base)
        assert np.array_equal(g.kappa(), want), n
    # the disc helper the solver tests use agrees with the pattern
    assert np.array_equal(oracle.disc_kappa(512, [[12.0, 0.5, 0.5, 0.3]], 1.0),
                          oracle.pattern_kappa(512, [], [[12.0, 0.5, 0.5, 0.3]], 1.0))
