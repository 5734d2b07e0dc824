"""The C restatement (oracle/maxwell_oracle.c) against golden vectors that the
reference's own modules produced (tests/golden/gen_golden.py)."""
import numpy as np
import pytest

RTOL = 1e-12


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


@pytest.mark.parametrize("fx", ["ops_n8.npz", "ops_n16.npz"])
def test_edge_operator(oracle, golden, fx):
    g = golden(fx)
    n, xf, yf = int(g["n"]), complex(g["xf"]), complex(g["yf"])
    y = oracle.addeval_edge(n, g["kappa_seam"], xf, yf, float(g["alpha"]), float(g["beta"]), g["x"], g["y"])
    assert rel(y, g["addeval"]) < RTOL
    e = oracle.energyprod_edge(n, g["kappa_seam"], xf, yf, 1.0, 1.0, g["x"], g["y"])
    m = oracle.massprod_edge(n, xf, yf, g["x"], g["y"])
    assert abs(e - g["products"][0]) / abs(g["products"][0]) < RTOL
    assert abs(m - g["products"][1]) / abs(g["products"][1]) < RTOL


def test_dense_edge_any_kappa(oracle, golden):
    g = golden("ops_n8.npz")
    n = int(g["n"])
    a = oracle.dense_edge(n, g["kappa_gen"], complex(g["xf"]), complex(g["yf"]), 1.0, 1.0)
    assert rel(a, g["dense_edge"]) < RTOL
    # the assembled operator is Hermitian and equals the matrix-free one
    assert np.abs(a - a.conj().T).max() < 1e-12 * np.abs(a).max()
    x = g["x"]
    y = oracle.addeval_edge(n, g["kappa_gen"], complex(g["xf"]), complex(g["yf"]), 1.0, 1.0, x, np.zeros_like(x))
    assert rel(y, a @ x) < RTOL


@pytest.mark.parametrize("fx", ["ops_n8.npz", "ops_n16.npz"])
@pytest.mark.parametrize("d,name", [(0, "fwd"), (1, "bwd"), (2, "symm")])
def test_afw_smoother(oracle, golden, fx, d, name):
    g = golden(fx)
    n = int(g["n"])
    x = oracle.gs_edge(n, g["kappa_gen"], complex(g["xf"]), complex(g["yf"]), 1.0, 1.0, d, g["b"], g["x"])
    assert rel(x, g[f"gs_{name}"]) < 1e-11


@pytest.mark.parametrize("fx", ["ops_n8.npz", "ops_n16.npz"])
def test_transfers_and_node_ops(oracle, golden, fx):
    g = golden(fx)
    n, xf, yf = int(g["n"]), complex(g["xf"]), complex(g["yf"])
    nc = n // 2
    assert rel(oracle.prolong_edge(nc, xf, yf, 1.0, g["c"], g["x"]), g["prolong"]) < RTOL
    assert rel(oracle.restrict_edge(nc, xf, yf, 1.0, g["x"], g["c"]), g["restrict"]) < RTOL
    assert rel(oracle.prolong_node(nc, xf, yf, 1.0, g["vc"], g["v"]), g["nprolong"]) < RTOL
    assert rel(oracle.restrict_node(nc, xf, yf, 1.0, g["v"], g["vc"]), g["nrestrict"]) < RTOL
    assert rel(oracle.addeval_node(n, xf, yf, 0.9, g["v"], g["w"]), g["naddeval"]) < RTOL
    for d, name in ((0, "fwd"), (1, "bwd"), (2, "symm")):
        assert rel(oracle.gs_node(n, xf, yf, 1.0, d, g["v"], g["w"]), g[f"ngs_{name}"]) < 1e-12
    assert rel(oracle.gradient(n, xf, yf, 1.0, g["v"], g["x"]), g["gradient"]) < RTOL
    assert rel(oracle.adjgradient(n, xf, yf, 1.0, g["x"], g["v"]), g["adjgradient"]) < RTOL
    assert rel(oracle.center_edge(n, g["x"]), g["center"]) < RTOL


def test_dense_node_and_coarsening(oracle, golden):
    g = golden("ops_n8.npz")
    n, xf, yf = int(g["n"]), complex(g["xf"]), complex(g["yf"])
    assert rel(oracle.dense_node(n, 1.0, 1.0, 1), g["dense_node_gamma"]) < RTOL
    assert rel(oracle.dense_node(n, xf, yf, 1), g["dense_node_k"]) < RTOL
    k = g["kappa_gen"]
    levels = [k]
    while len(levels) < 3:
        levels.append(oracle.coarsen_kappa(int(np.sqrt(levels[-1].size)), levels[-1]))
    assert rel(np.concatenate(levels), g["coarsen"]) < RTOL


def test_vcycles_and_pinvit(oracle, golden):
    g = golden("vcycle_n16.npz")
    n0, L, xf, yf = int(g["n0"]), int(g["L"]), complex(g["xf"]), complex(g["yf"])
    b, bn = g["b"], g["bn"]
    x = oracle.vcycle_edge(n0, L, g["kappa"], xf, yf, 2, 1, 2, b, np.zeros_like(b))
    assert rel(x, g["vcycle_edge"]) < 1e-10
    x = oracle.vcycle_edge(n0, L, g["kappa"], xf, yf, 2, 0, 1, b, np.zeros_like(b))
    assert rel(x, g["vcycle_edge_nocoarse"]) < 1e-10
    x = oracle.vcycle_node(n0, L, xf, yf, 2, 1, 3, bn, np.zeros_like(bn))
    assert rel(x, g["vcycle_node"]) < 1e-10
    x = oracle.vcycle_node(n0, L, 1.0, 1.0, 2, 1, 3, bn, np.zeros_like(bn))
    assert rel(x, g["vcycle_node_gamma"]) < 1e-10


def test_dense_eigensolvers(oracle):
    rng = np.random.default_rng(5)
    n = 24
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    a = a + a.conj().T
    w, v = oracle.heev(np.tril(a))
    assert np.allclose(np.sort(np.linalg.eigvalsh(a)), w, rtol=0, atol=1e-12 * np.abs(w).max())
    assert np.abs(a @ v - v * w).max() < 1e-11 * np.abs(w).max()
    b = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    b = b @ b.conj().T + n * np.eye(n)
    info, w2, x = oracle.hegv(np.tril(a), np.tril(b))
    assert info == 0
    assert np.abs(a @ x - b @ x * w2).max() < 1e-10 * np.abs(w2).max()
    assert np.abs(x.conj().T @ b @ x - np.eye(n)).max() < 1e-11


def test_block_pinvit_matches_reference_eigenvalues(oracle, golden):
    """Same flow as the reference's exp_bloch2d (nested iteration, warm
    start, PINVIT + Ritz, absolute defect <= 1e-9): eigenvalues agree to the
    stated 1e-8 relative tolerance (in practice ~1e-15)."""
    g = golden("eigs_n32_disc.npz")
    st, lam, steps, res, _ = oracle.bloch_solve(
        g["kappa"], g["factors"], n0=int(g["n0"]), L=int(g["L"]), ieigs=int(g["ieigs"]), m=int(g["m"]),
        method=0, max_nested=80, max_steps=80, tol=float(g["tol"]), relative=0, extrapolation="2", wave=1)
    assert st == 0
    ie = int(g["ieigs"])
    assert np.abs(lam[:, :ie] - g["lam"][:, :ie]).max() / g["lam"][:, :ie].max() < 1e-8
    assert res[:, :ie].max() <= float(g["tol"])


def test_lobpcg_matches_reference_eigenvalues(oracle, golden):
    g = golden("eigs_n32_disc.npz")
    st, lam, steps, res, _ = oracle.bloch_solve(
        g["kappa"], g["factors"], n0=int(g["n0"]), L=int(g["L"]), ieigs=int(g["ieigs"]), m=int(g["m"]),
        method=1, max_nested=40, max_steps=40, tol=float(g["tol"]), relative=0, extrapolation="2", wave=1)
    assert st == 0
    ie = int(g["ieigs"])
    assert np.abs(lam[:, :ie] - g["lam"][:, :ie]).max() / g["lam"][:, :ie].max() < 1e-8
    assert steps.max() < 30


def test_pinvit_single_vector(oracle, golden):
    """One pinvit_edge2d step (edge2d.c:6298-6328) composed from the restated
    operators: defect, two edge V-cycles, update, gradient lifting."""
    g = golden("vcycle_n16.npz")
    n0, L, xf, yf = int(g["n0"]), int(g["L"]), complex(g["xf"]), complex(g["yf"])
    n = n0 << L
    e = g["e"].copy()
    b = oracle.addeval_edge(n, g["kappa"], xf, yf, 1.0, 1.0 - 40.0, e, np.zeros_like(e))
    x = oracle.vcycle_edge(n0, L, g["kappa"], xf, yf, 2, 1, 2, b, np.zeros_like(b))
    e -= x
    d = oracle.addeval_edge(n, g["kappa"], xf, yf, 0.0, 1.0, e, np.zeros_like(e))
    bg = oracle.adjgradient(n, xf, yf, 1.0, d, np.zeros(n * n, complex))
    xg = oracle.vcycle_node(n0, L, xf, yf, 2, 1, 5, bg, np.zeros_like(bg))
    e = oracle.gradient(n, xf, yf, -1.0, xg, e)
    assert rel(e, g["pinvit"]) < 1e-10


def test_oracle_adjoint_matches_finite_differences(oracle):
    """The CPU reference gradient (om_eps_sensitivity on the oracle's own
    M-normalised eigenvectors) against central differences of the oracle's
    eigenvalues, step 1e-6 relative on eps of single cells: 1e-5 relative."""
    n0, L = 8, 1
    n = n0 << L
    rng = np.random.default_rng(3)
    eps = 1.0 + 11.0 * rng.random(n * n)
    fac = np.array([[np.exp(0.9j), np.exp(0.4j)]])

    def solve(e, vectors=False):
        st, lam, _, res, vec = oracle.bloch_solve(1.0 / e, fac, n0=n0, L=L, ieigs=6, m=8, method=1, max_nested=60,
                                                  max_steps=100, tol=1e-11, relative=1, extrapolation="n",
                                                  wave=1, want_vectors=vectors)
        assert st == 0 and res[:, :6].max() <= 1e-11
        return lam, vec

    lam, vec = solve(eps, True)
    band = 1
    assert abs(lam[0, band] - lam[0, band - 1]) > 1e-6 and abs(lam[0, band + 1] - lam[0, band]) > 1e-6
    w = np.zeros(8)
    w[band] = 1.0
    g = oracle.eps_sensitivity(n, 1.0 / eps, *fac[0], vec[0], w)
    for c in (5, 77, 200):
        h = 1e-6 * eps[c]
        ep, em = eps.copy(), eps.copy()
        ep[c] += h
        em[c] -= h
        fd = (solve(ep)[0][0, band] - solve(em)[0][0, band]) / (2 * h)
        assert abs(fd - g[c]) <= 1e-5 * np.abs(g).max(), (c, fd, g[c])


def test_oracle_colour_smoother_converges(oracle, golden):
    """The four-colour patch smoother (the GPU solver's order) is a convergent
    splitting of alpha A + beta M: symmetric sweeps shrink the error of
    (A + M) x = b in the energy norm, every sweep."""
    g = golden("ops_n16.npz")
    n, kap, xf, yf = int(g["n"]), g["kappa_gen"], complex(g["xf"]), complex(g["yf"])
    rng = np.random.default_rng(4)
    xs = rng.standard_normal(2 * n * n) + 1j * rng.standard_normal(2 * n * n)
    b = oracle.addeval_edge(n, kap, xf, yf, 1.0, 1.0, xs, np.zeros_like(xs))
    x = np.zeros_like(xs)

    def energy(e):
        return np.real(np.vdot(e, oracle.addeval_edge(n, kap, xf, yf, 1.0, 1.0, e, np.zeros_like(e))))

    last = energy(x - xs)
    for _ in range(6):
        x = oracle.gs_edge_colour(n, kap, xf, yf, 1.0, 1.0, 2, b, x)
        cur = energy(x - xs)
        assert cur < 0.9 * last
        last = cur


def driver_curve_reference(g):
    """Per point of the reference driver's curve, the converged eigenvalues
    of its protocol (the first ieigs) without Gamma's two harmonic zero
    modes, which the driver keeps and the constant-field removal here takes
    out."""
    ie = int(g["ieigs"])
    return [row[:ie][np.abs(row[:ie]) > 1e-3] for row in g["lam"]]


def test_oracle_matches_reference_driver_curve(oracle, golden):
    """The reference's own driver program (exp_bloch2d: Kivshar disc, 16^2,
    4 steps per edge of its Gamma-X-M-Gamma curve, block PINVIT to the
    absolute residual 1e-8): the oracle's eigenvalues at the same points
    agree with its protocol file to the file's 6 decimals."""
    g = golden("bloch_curve_n16_kivshar.npz")
    n0, L = int(g["n0"]), int(g["L"])
    kap = oracle.disc_kappa(n0 << L, [g["disc"]], float(g["eps_base"]))
    st, lam, steps, res, _ = oracle.bloch_solve(
        kap, g["factors"], n0=n0, L=L, ieigs=int(g["ieigs"]), m=int(g["m"]), method=0, max_nested=40,
        max_steps=80, tol=float(g["tol"]), relative=0, extrapolation="2", wave=1)
    assert st == 0
    for k, ref in enumerate(driver_curve_reference(g)):
        assert np.abs(lam[k, :len(ref)] - ref).max() < 2e-6, (k, lam[k, :len(ref)], ref)


def test_oracle_point_smoother_and_hiptmair_cycle(oracle, golden):
    """The restated point smoother (gs*_simple_edge2d) and Hiptmair cycle
    (hcycle_edge2d) against the reference's golden vectors."""
    g = golden("hiptmair_n16.npz")
    n0, L = int(g["n0"]), int(g["L"])
    n = n0 << L
    xf, yf = complex(g["xf"]), complex(g["yf"])
    for d, name in ((0, "fwd"), (1, "bwd"), (2, "symm")):
        got = oracle.gs_edge_simple(n, g["kappa"], xf, yf, 1.0, 1.0, d, g["b"], g["x"])
        assert np.abs(got - g["simple_" + name]).max() < 1e-12 * np.abs(g["simple_" + name]).max()
    for key, coarse, cycles in (("hcycle", 1, 2), ("hcycle_nocoarse", 0, 1)):
        got = oracle.hcycle_edge(n0, L, g["kappa"], xf, yf, 2, coarse, cycles, g["b"], np.zeros_like(g["b"]))
        assert np.abs(got - g[key]).max() < 1e-11 * np.abs(g[key]).max(), key
