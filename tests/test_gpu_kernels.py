"""CUDA kernels through the C ABI against the oracle restatement, batched over
k-points and vectors.  Tolerances: FP64 storage 1e-12 relative, float-float
storage 1e-12, FP32 storage 2e-5 (the kernels compute in the storage's
arithmetic)."""
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
    rng = np.random.default_rng(11)
    n, K, m = 16, 3, 3
    kap = 1.0 / (1.0 + 11.0 * rng.random(n * n))
    return rng, n, K, m, kap


@pytest.mark.parametrize("prec", [mx.C128, mx.CDD, mx.C64])
def test_edge_operator(oracle, setup, prec):
    rng, n, K, m, kap = setup
    g = mx.Grid(n, K, kap, FACTORS)
    x, y = cv(rng, K, m, 2 * n * n), cv(rng, K, m, 2 * n * n)
    ex, ey = mx.Edge(g, m, prec, x), mx.Edge(g, m, prec, y)
    mx.check(mx.lib().addeval_edge2d_gpu(mx.fz(1.3), mx.fz(0.7), ex.h, ey.h))
    got = ey.get()
    want = np.array([[oracle.addeval_edge(n, kap, *FACTORS[k], 1.3, 0.7, x[k, v], y[k, v]) for v in range(m)]
                     for k in range(K)])
    assert rel(got, want) < TOL[prec]


@pytest.mark.parametrize("prec", [mx.C128, mx.CDD, mx.C64])
def test_shifted_operator_and_products(oracle, setup, prec):
    """The operator with one shift per vector and the energy and mass
    products in each storage precision (the solver's blocks are c64 and
    float-float)."""
    rng, n, K, m, kap = setup
    tol = TOL[prec]
    g = mx.Grid(n, K, kap, FACTORS)
    x, y = cv(rng, K, m, 2 * n * n), cv(rng, K, m, 2 * n * n)
    beta = rng.random((K, m))
    ex, ey = mx.Edge(g, m, prec, x), mx.Edge(g, m, prec, y)
    x, y = ex.get(), ey.get()   # the values as stored
    mx.check(mx.lib().addeval_shifted_edge2d_gpu(1.0, mx._ptr(np.ascontiguousarray(beta)), ex.h, ey.h))
    want = np.array([[oracle.addeval_edge(n, kap, *FACTORS[k], 1.0, beta[k, v], x[k, v], y[k, v]) for v in range(m)]
                     for k in range(K)])
    assert rel(ey.get(), want) < tol
    ey.put(y)
    out = np.zeros(K * m, np.complex128)
    mx.check(mx.lib().energyprod_edge2d_gpu(mx.fz(1.0), mx.fz(1.0), ex.h, ey.h, mx._ptr(out)))
    want = np.array([[oracle.energyprod_edge(n, kap, *FACTORS[k], 1.0, 1.0, x[k, v], y[k, v]) for v in range(m)]
                     for k in range(K)]).reshape(-1)
    # energyprod returns x^H K y for Hermitian K (edge2d.c:1958)
    assert np.abs(out - want).max() / np.abs(want).max() < tol
    mx.check(mx.lib().massprod_edge2d_gpu(ex.h, ey.h, mx._ptr(out)))
    want = np.array([[oracle.massprod_edge(n, *FACTORS[k], x[k, v], y[k, v]) for v in range(m)]
                     for k in range(K)]).reshape(-1)
    assert np.abs(out - want).max() / np.abs(want).max() < tol


@pytest.mark.parametrize("prec", [mx.C128, mx.C64])
@pytest.mark.parametrize("direction", [0, 1, 2])
def test_afw_smoother(oracle, setup, prec, direction):
    rng, n, K, m, kap = setup
    g = mx.Grid(n, K, kap, FACTORS)
    b, x = cv(rng, K, m, 2 * n * n), cv(rng, K, m, 2 * n * n)
    eb, ex = mx.Edge(g, m, prec, b), mx.Edge(g, m, prec, x)
    fn = [mx.lib().gsforward_edge2d_gpu, mx.lib().gsbackward_edge2d_gpu, mx.lib().gssymm_edge2d_gpu][direction]
    mx.check(fn(mx.fz(1.0), mx.fz(1.0), eb.h, ex.h))
    want = np.array([[oracle.gs_edge(n, kap, *FACTORS[k], 1.0, 1.0, direction, b[k, v], x[k, v]) for v in range(m)]
                     for k in range(K)])
    assert rel(ex.get(), want) < (1e-11 if prec == mx.C128 else 1e-4)


@pytest.mark.parametrize("n, m, prec", [(16, 4, mx.C64), (80, 4, mx.C64), (256, 16, mx.C64), (128, 16, mx.C128),
                                         (128, 16, mx.CDD), (32, 1, mx.C64), (48, 7, mx.C64), (24, 7, mx.C128),
                                         (128, 12, mx.C64), (512, 4, mx.C64)])
@pytest.mark.parametrize("direction", [0, 1, 2])
def test_node_gs_even_block(oracle, n, m, prec, direction):
    """Node Gauss-Seidel against the oracle: a row in one segment (n = 16,
    80 at 4 vectors) and in several with a partial last one (n = 256 at 16
    c64 vectors: segments of 112 positions; n = 128 at 16 FP64 or
    float-float vectors: segments of 48); one vector and 7 vectors (lane
    groups that leave part of a warp idle)."""
    rng = np.random.default_rng(5)
    K = 3
    g = mx.Grid(n, K, None, FACTORS)
    v_, w_ = cv(rng, K, m, n * n), cv(rng, K, m, n * n)
    nv, nw = mx.Node(g, m, prec, v_), mx.Node(g, m, prec, w_)
    fn = [mx.lib().gsforward_node2d_gpu, mx.lib().gsbackward_node2d_gpu, mx.lib().gssymm_node2d_gpu][direction]
    mx.check(fn(mx.fz(1.0), nv.h, nw.h))
    want = np.array([[oracle.gs_node(n, *FACTORS[k], 1.0, direction, v_[k, i], w_[k, i]) for i in range(m)]
                     for k in range(K)])
    assert rel(nw.get(), want) < (2e-5 if prec == mx.C64 else 1e-11)


@pytest.mark.parametrize("strip, band", [(64, 1), (64, 5), (128, 3), (128, 64)])
@pytest.mark.parametrize("direction", [0, 1, 2])
def test_node_gs_tiled_shapes(oracle, strip, band, direction):
    """The tiled out-of-place node sweep (c64 blocks, m a multiple of 4,
    n >= 128) under several strip widths and band heights -- bands of one
    pair, bands that do not divide the (n-2)/2 pairs, a band taller than
    the grid -- against the oracle's in-place sweep: the strips at both
    ends wrap through the seam, the first band reads the new row 0 and the
    last one the old row n-1."""
    rng = np.random.default_rng(11)
    n, m, K = 256, 8, 3
    default = mx.get_tuning()
    try:
        mx.set_tuning(**dict(default, node_strip=strip, node_band=band))
        g = mx.Grid(n, K, None, FACTORS)
        v_, w_ = cv(rng, K, m, n * n), cv(rng, K, m, n * n)
        nv, nw = mx.Node(g, m, mx.C64, v_), mx.Node(g, m, mx.C64, w_)
        fn = [mx.lib().gsforward_node2d_gpu, mx.lib().gsbackward_node2d_gpu, mx.lib().gssymm_node2d_gpu][direction]
        mx.check(fn(mx.fz(0.7), nv.h, nw.h))
    finally:
        mx.set_tuning(**default)
    want = np.array([[oracle.gs_node(n, *FACTORS[k], 0.7, direction, v_[k, i], w_[k, i]) for i in range(m)]
                     for k in range(K)])
    assert rel(nw.get(), want) < 2e-5


@pytest.mark.parametrize("prec", [mx.C128, mx.CDD, mx.C64])
@pytest.mark.parametrize("direction", [0, 1, 2])
def test_colour_smoother(oracle, setup, prec, direction):
    """The four-colour patch smoother (gscolour_edge2d_gpu) against the
    oracle's restatement of the same order."""
    rng, n, K, m, kap = setup
    g = mx.Grid(n, K, kap, FACTORS)
    b, x = cv(rng, K, m, 2 * n * n), cv(rng, K, m, 2 * n * n)
    eb, ex = mx.Edge(g, m, prec, b), mx.Edge(g, m, prec, x)
    mx.check(mx.lib().gscolour_edge2d_gpu(mx.fz(1.0), mx.fz(1.0), eb.h, ex.h, direction))
    want = np.array([[oracle.gs_edge_colour(n, kap, *FACTORS[k], 1.0, 1.0, direction, b[k, v], x[k, v])
                      for v in range(m)] for k in range(K)])
    assert rel(ex.get(), want) < (1e-11 if prec != mx.C64 else 1e-4)


@pytest.mark.parametrize("n, m", [(16, 1), (24, 7)])
@pytest.mark.parametrize("prec", [mx.C128, mx.C64])
@pytest.mark.parametrize("direction", [0, 1])
def test_colour_smoother_block_sizes(oracle, n, m, prec, direction):
    """The colour smoother with one vector and with 7 (patch lanes per CTA
    256 / m), against the oracle's restatement of the same order."""
    rng = np.random.default_rng(17)
    K = 2
    kap = 1.0 / (1.0 + 11.0 * rng.random(n * n))
    g = mx.Grid(n, K, kap, FACTORS[:K])
    b, x = cv(rng, K, m, 2 * n * n), cv(rng, K, m, 2 * n * n)
    eb, ex = mx.Edge(g, m, prec, b), mx.Edge(g, m, prec, x)
    mx.check(mx.lib().gscolour_edge2d_gpu(mx.fz(1.0), mx.fz(1.0), eb.h, ex.h, direction))
    want = np.array([[oracle.gs_edge_colour(n, kap, *FACTORS[k], 1.0, 1.0, direction, b[k, v], x[k, v])
                      for v in range(m)] for k in range(K)])
    assert rel(ex.get(), want) < (1e-11 if prec == mx.C128 else 1e-4)


@pytest.mark.parametrize("smoother", [0, 1])
def test_solver_smoothers_agree(oracle, smoother):
    """Both edge smoothers drive the mixed LOBPCG to the same eigenvalues."""
    n0, L = 8, 2
    n = n0 << L
    kap = oracle.disc_kappa(n, [[12.0, 0.5, 0.5, 0.3]], 1.0)
    fac = np.array([[np.exp(0.4j), np.exp(1.1j)], [np.exp(2.5j), 1.0]])
    s = mx.Solver(kap, n0=n0, L=L, ieigs=8, m=12, method=1, precision=1, wave=2, relative=1, tol=1e-9,
                  max_nested=5, max_steps=60, smoother=smoother)
    lam, steps, res = s.solve(fac)
    st, lam_o, _, _, _ = oracle.bloch_solve(kap, fac, n0=n0, L=L, ieigs=8, m=12, method=1, max_nested=40,
                                            max_steps=60, tol=1e-9, relative=1, extrapolation="n", wave=2)
    assert res[:, :8].max() <= 1e-9
    assert np.abs(lam[:, :8] - lam_o[:, :8]).max() / lam_o[:, :8].max() < 1e-8


@pytest.mark.parametrize("n", [44, 64])
@pytest.mark.parametrize("prec", [mx.C128, mx.CDD, mx.C64])
@pytest.mark.parametrize("strips", [True, False])
def test_residual_restriction_strips(oracle, n, prec, strips):
    """The fused node residual + restriction in both forms: a thread per
    coarse node, and (forced here by restrict_strip_log2 = 0) strips of 8
    coarse rows -- coarse grids of 22 and 32 rows hold strips inside the
    cell (no seam test), strips along the seam and a ragged last strip."""
    rng = np.random.default_rng(n)
    K, m, nc = 3, 3, n // 2
    kap = 1.0 / (1.0 + 11.0 * rng.random(n * n))
    gf = mx.Grid(n, K, kap, FACTORS)
    gc = gf.coarsen()
    x, b, c = cv(rng, K, m, n * n), cv(rng, K, m, n * n), cv(rng, K, m, nc * nc)
    nx, nb, nco = mx.Node(gf, m, prec, x), mx.Node(gf, m, prec, b), mx.Node(gc, m, prec, c)
    default = mx.get_tuning()
    try:
        mx.set_tuning(**dict(default, restrict_strip_log2=0 if strips else 62))
        mx.check(mx.lib().residual_restriction_node2d_gpu(mx.fz(0.8), nb.h, nx.h, nco.h))
    finally:
        mx.set_tuning(**default)
    want = np.array([[oracle.restrict_node(nc, *FACTORS[k], 1.0,
                                           oracle.addeval_node(n, *FACTORS[k], -0.8, x[k, i], b[k, i]),
                                           np.zeros(nc * nc)) for i in range(m)] for k in range(K)])
    assert rel(nco.get(), want) < TOL[prec] * 10


@pytest.mark.parametrize("prec", [mx.C128, mx.C64])
def test_transfers_node_ops_gradient(oracle, setup, prec):
    rng, n, K, m, kap = setup
    nc = n // 2
    gf = mx.Grid(n, K, kap, FACTORS)
    gc = gf.coarsen()
    tol = TOL[prec] * 10
    c, f = cv(rng, K, m, 2 * nc * nc), cv(rng, K, m, 2 * n * n)
    ec, ef = mx.Edge(gc, m, prec, c), mx.Edge(gf, m, prec, f)
    mx.check(mx.lib().prolongation_edge2d_gpu(mx.fz(1.0), ec.h, ef.h))
    want = np.array([[oracle.prolong_edge(nc, *FACTORS[k], 1.0, c[k, v], f[k, v]) for v in range(m)] for k in range(K)])
    assert rel(ef.get(), want) < tol
    ef.put(f)
    mx.check(mx.lib().restriction_edge2d_gpu(mx.fz(1.0), ef.h, ec.h))
    want = np.array([[oracle.restrict_edge(nc, *FACTORS[k], 1.0, f[k, v], c[k, v]) for v in range(m)] for k in range(K)])
    assert rel(ec.get(), want) < tol
    v_, w_ = cv(rng, K, m, n * n), cv(rng, K, m, n * n)
    vc = cv(rng, K, m, nc * nc)
    nv, nw, nvc = mx.Node(gf, m, prec, v_), mx.Node(gf, m, prec, w_), mx.Node(gc, m, prec, vc)
    mx.check(mx.lib().addeval_node2d_gpu(mx.fz(0.9), nv.h, nw.h))
    want = np.array([[oracle.addeval_node(n, *FACTORS[k], 0.9, v_[k, i], w_[k, i]) for i in range(m)] for k in range(K)])
    assert rel(nw.get(), want) < tol
    for d, fn in enumerate([mx.lib().gsforward_node2d_gpu, mx.lib().gsbackward_node2d_gpu, mx.lib().gssymm_node2d_gpu]):
        nw.put(w_)
        mx.check(fn(mx.fz(1.0), nv.h, nw.h))
        want = np.array([[oracle.gs_node(n, *FACTORS[k], 1.0, d, v_[k, i], w_[k, i]) for i in range(m)] for k in range(K)])
        assert rel(nw.get(), want) < tol * 10
    mx.check(mx.lib().prolongation_node2d_gpu(mx.fz(1.0), nvc.h, nv.h))
    want = np.array([[oracle.prolong_node(nc, *FACTORS[k], 1.0, vc[k, i], v_[k, i]) for i in range(m)] for k in range(K)])
    assert rel(nv.get(), want) < tol
    nv.put(v_)
    mx.check(mx.lib().restriction_node2d_gpu(mx.fz(1.0), nv.h, nvc.h))
    want = np.array([[oracle.restrict_node(nc, *FACTORS[k], 1.0, v_[k, i], vc[k, i]) for i in range(m)] for k in range(K)])
    assert rel(nvc.get(), want) < tol
    # the V-cycle's fused residual + restriction: c = R(b - 0.8 L x), c overwritten
    nw.put(w_)
    mx.check(mx.lib().residual_restriction_node2d_gpu(mx.fz(0.8), nw.h, nv.h, nvc.h))
    want = np.array([[oracle.restrict_node(nc, *FACTORS[k], 1.0,
                                           oracle.addeval_node(n, *FACTORS[k], -0.8, v_[k, i], w_[k, i]),
                                           np.zeros(nc * nc)) for i in range(m)] for k in range(K)])
    assert rel(nvc.get(), want) < tol
    ef.put(f)
    mx.check(mx.lib().gradient_node2d_gpu(mx.fz(-1.0), nv.h, ef.h))
    want = np.array([[oracle.gradient(n, *FACTORS[k], -1.0, v_[k, i], f[k, i]) for i in range(m)] for k in range(K)])
    assert rel(ef.get(), want) < tol
    ef.put(f)
    nv.put(v_)
    mx.check(mx.lib().adjgradient_node2d_gpu(mx.fz(1.0), ef.h, nv.h))
    want = np.array([[oracle.adjgradient(n, *FACTORS[k], 1.0, f[k, i], v_[k, i]) for i in range(m)] for k in range(K)])
    assert rel(nv.get(), want) < tol


def test_dense_and_coarse_solvers(oracle, setup):
    rng, _, K, _, _ = setup
    n = 8
    kap = 1.0 / (1.0 + 11.0 * rng.random(n * n))
    g = mx.Grid(n, K, kap, FACTORS)
    N = 2 * n * n
    A = mx.Matrix(N, K)
    mx.check(mx.lib().densematrix_edge2d_gpu(mx.fz(1.0), mx.fz(1.0), g.h, A.h))
    got = A.get()
    for k in range(K):
        want = oracle.dense_edge(n, kap, *FACTORS[k], 1.0, 1.0)
        assert rel(got[k], want) < 1e-13
    info = np.zeros(K, np.int32)
    mx.check(mx.lib().potrf_matrix_gpu(A.h, mx._ptr(info)))
    assert (info == 0).all()
    inv = A.get()
    for k in range(K):
        want = oracle.dense_edge(n, kap, *FACTORS[k], 1.0, 1.0)
        assert np.abs(inv[k] @ want - np.eye(N)).max() < 1e-10
    Nn = n * n
    An = mx.Matrix(Nn, K)
    mx.check(mx.lib().densematrix_node2d_gpu(1, g.h, An.h))
    got = An.get()
    for k in range(K):
        assert rel(got[k], oracle.dense_node(n, *FACTORS[k], 1)) < 1e-13
    # generalized eigenproblem of the coarse curl-curl and mass (exp_bloch2d.c:530-554)
    Aa, Mm = mx.Matrix(N, K), mx.Matrix(N, K)
    mx.check(mx.lib().densematrix_edge2d_gpu(mx.fz(1.0), mx.fz(0.0), g.h, Aa.h))
    mx.check(mx.lib().densematrix_edge2d_gpu(mx.fz(0.0), mx.fz(1.0), g.h, Mm.h))
    lam = np.zeros(K * N)
    mx.check(mx.lib().sygv_matrix_gpu(Aa.h, Mm.h, mx._ptr(lam), mx._ptr(info)))
    assert (info == 0).all()
    lam = lam.reshape(K, N)
    for k in range(K):
        info_o, w, _ = oracle.hegv(oracle.dense_edge(n, kap, *FACTORS[k], 1.0, 0.0),
                                   oracle.dense_edge(n, kap, *FACTORS[k], 0.0, 1.0))
        assert np.abs(lam[k] - w).max() < 1e-9 * np.abs(w).max()


@pytest.mark.parametrize("prec", [mx.C128, mx.CDD, mx.C64])
def test_vcycles_match_oracle(oracle, golden, prec):
    """Edge and node V-cycles against the reference's own (golden vectors),
    in each storage precision; c64 is the solver's multigrid arithmetic and
    lands within its rounding (1e-4 relative after two and three cycles)."""
    tol = 1e-4 if prec == mx.C64 else 1e-10
    g0 = golden("vcycle_n16.npz")
    n0, L, xf, yf = int(g0["n0"]), int(g0["L"]), complex(g0["xf"]), complex(g0["yf"])
    kap = g0["kappa"]
    grids = [mx.Grid(n0 << L, 1, kap, [[xf, yf]])]
    for _ in range(L):
        grids.append(grids[-1].coarsen())
    grids = grids[::-1]
    b = [mx.Edge(gr, 1, prec) for gr in grids]
    x = [mx.Edge(gr, 1, prec) for gr in grids]
    d = [mx.Edge(gr, 1, prec) for gr in grids]
    b[L].put(g0["b"])
    Ac = mx.Matrix(2 * n0 * n0, 1)
    mx.check(mx.lib().densematrix_edge2d_gpu(mx.fz(1.0), mx.fz(1.0), grids[0].h, Ac.h))
    info = np.zeros(1, np.int32)
    mx.check(mx.lib().potrf_matrix_gpu(Ac.h, mx._ptr(info)))
    arr = lambda objs: (mx.C.c_void_p * len(objs))(*[o.h for o in objs])
    import ctypes as C
    for _ in range(2):
        mx.check(mx.lib().vcycle_edge2d_gpu(L, 2, Ac.h, C.cast(arr(b), C.c_void_p), C.cast(arr(x), C.c_void_p),
                                            C.cast(arr(d), C.c_void_p)))
    assert rel(x[L].get()[0, 0], g0["vcycle_edge"]) < tol
    nb = [mx.Node(gr, 1, prec) for gr in grids]
    nx = [mx.Node(gr, 1, prec) for gr in grids]
    nd = [mx.Node(gr, 1, prec) for gr in grids]
    nb[L].put(g0["bn"])
    An = mx.Matrix(n0 * n0, 1)
    mx.check(mx.lib().densematrix_node2d_gpu(1, grids[0].h, An.h))
    mx.check(mx.lib().potrf_matrix_gpu(An.h, mx._ptr(info)))
    for _ in range(3):
        mx.check(mx.lib().vcycle_node2d_gpu(L, 2, An.h, C.cast(arr(nb), C.c_void_p), C.cast(arr(nx), C.c_void_p),
                                            C.cast(arr(nd), C.c_void_p)))
    assert rel(nx[L].get()[0, 0], g0["vcycle_node"]) < tol


def test_center(oracle, setup):
    rng, n, K, m, kap = setup
    g = mx.Grid(n, K, kap, FACTORS)
    x = cv(rng, K, m, 2 * n * n)
    e = mx.Edge(g, m, mx.C128, x)
    mx.check(mx.lib().center_edge2d_gpu(e.h))
    want = np.array([[oracle.center_edge(n, x[k, v]) for v in range(m)] for k in range(K)])
    assert rel(e.get(), want) < 1e-13
