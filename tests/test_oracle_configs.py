"""The oracle and the benchmark's inputs at the task's configurations (CPU).

* The permittivity fixtures record the cell count inside the disc and the
  sum of 1/eps; the oracle's rasterisation (setpattern_grid2d's rule) and
  the benchmark's own (bench.disc_kappa) reproduce them exactly.
* The oracle restatement's LOBPCG reproduces the reference's own block
  PINVIT eigenvalues of config 1 (64^2, tests/golden/config1_n64_disc.npz)
  at two k-points to 1e-8 relative.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


@pytest.mark.parametrize("name", ["config1_n64_disc.npz", "headline_n512_disc.npz"])
def test_fixture_permittivity(oracle, golden, name):
    g = golden(name)
    n = int(g["n0"]) << int(g["L"])
    kap = oracle.disc_kappa(n, [g["disc"]], float(g["eps_base"]))
    assert int((kap < 1.0).sum()) == int(g["inside"])
    assert kap.sum() == pytest.approx(float(g["kappa_sum"]), rel=1e-15)
    if name.startswith("headline"):
        import bench
        assert np.array_equal(bench.disc_kappa(n), kap)


def test_oracle_matches_config1_reference(oracle, golden):
    g = golden("config1_n64_disc.npz")
    n0, L, ie, m = int(g["n0"]), int(g["L"]), int(g["ieigs"]), int(g["m"])
    kap = oracle.disc_kappa(n0 << L, [g["disc"]], float(g["eps_base"]))
    pick = [3, 11]
    st, lam, steps, res, _ = oracle.bloch_solve(kap, g["factors"][pick], n0=n0, L=L, ieigs=ie, m=m, method=1,
                                                max_nested=40, max_steps=80, tol=1e-10, relative=1,
                                                extrapolation="n", wave=1)
    assert st == 0
    want = g["lam"][pick, :ie]
    assert (np.abs(lam[:, :ie] - want) / want).max() < 1e-8


@pytest.fixture(scope="module")
def driver_curve(oracle, golden):
    """The oracle's solve of the reference driver's 16^2 Kivshar curve
    (Gamma-X-M-Gamma, 4 steps per edge) with its eigenvectors."""
    g = golden("bloch_curve_n16_kivshar.npz")
    n0, L, ie, m = int(g["n0"]), int(g["L"]), int(g["ieigs"]), int(g["m"])
    n = n0 << L
    kap = oracle.disc_kappa(n, [g["disc"]], float(g["eps_base"]))
    fac = g["factors"]
    st, lam, steps, res, vec = oracle.bloch_solve(kap, fac, n0=n0, L=L, ieigs=ie, m=m, method=1, max_nested=40,
                                                  max_steps=80, tol=1e-9, relative=0, extrapolation="n", wave=1,
                                                  want_vectors=True)
    assert st == 0
    nk = len(fac)
    vertex = np.array([1 if p in (0, 4, 8, nk - 1) else 0 for p in range(nk)], np.int32)
    return g, n, fac, ie, m, lam, vec, vertex


def test_chern_sums_do_not_depend_on_the_eigenvector_phases(oracle, driver_curve):
    """The sign continuity absorbs any phase of the input eigenvectors: Chern
    partial sums along the reference driver's curve are the same when every
    eigenvector of every point is multiplied by a random unit phase."""
    g, n, fac, ie, m, lam, vec, vertex = driver_curve
    nk = len(fac)
    _, _, ch1, _ = oracle.continuity(n, fac, ie, vertex, "s", ie, vec, lam)
    rng = np.random.default_rng(3)
    ph = np.exp(2j * np.pi * rng.random((nk, m)))[:, :, None]
    _, _, ch2, _ = oracle.continuity(n, fac, ie, vertex, "s", ie, vec * ph, lam)
    assert np.abs(ch1 - ch2).max() < 1e-12
    assert np.abs(ch1[1:]).max() > 1e-3       # the sums are not trivially zero


def test_chern_increments_match_the_driver_protocol(oracle, driver_curve):
    """Pin of the continuity restatement against the reference driver's own
    protocol file (exp_bloch2d.c:1058-1216, 1227-1235; the fixture keeps its
    6-decimal Chern partial sums).  The sums themselves are anchored on
    Gamma, where the driver keeps the two constant-field zero modes in an
    arbitrary basis, so they are compared as increments from point to point,
    on the stretches where the alignment does not reach back to Gamma: after
    the vertex X for the bands that stay simple (1st and 4th: the 2nd and
    3rd meet at M, 12.280956 twice), and on the X-M edge before M for all
    four.  Tolerance: two 6-decimal roundings."""
    g, n, fac, ie, m, lam, vec, vertex = driver_curve
    _, _, ch, _ = oracle.continuity(n, fac, ie, vertex, "s", ie, vec, lam)
    got, want = np.diff(ch, axis=0), np.diff(g["chern"], axis=0)   # row r: point r -> r + 1
    x_point, m_point = 4, 8
    assert np.isclose(g["lam"][m_point, 1], g["lam"][m_point, 2], rtol=1e-6)   # the degeneracy at M
    simple = [0, 3]
    d = np.abs(got[x_point:, simple] - want[x_point:, simple]).max()
    assert d < 3e-6, d
    d = np.abs(got[x_point:m_point - 1] - want[x_point:m_point - 1]).max()
    assert d < 3e-6, d
    assert np.abs(want[x_point:]).max() > 1e-2   # the compared increments are not trivially small


def test_oracle_matches_the_surface_driver(oracle, golden):
    """The restatement's eigenvalues on the reference surface driver's own
    full-zone grid (exp_blochsurf: Kivshar disc, 16^2, 4 x 4 k-points with
    k = 2 pi i / 3 - pi, absolute residual 1e-8; tests/golden/gen_blochsurf.py)
    agree with the driver's protocol to its 6 decimals.  The grid holds M,
    where the 2nd and 3rd bands meet, and no Gamma."""
    g = golden("blochsurf_n16_kivshar.npz")
    n0, L, ie, m = int(g["n0"]), int(g["L"]), int(g["ieigs"]), int(g["m"])
    kap = oracle.disc_kappa(n0 << L, [g["disc"]], float(g["eps_base"]))
    st, lam, steps, res, _ = oracle.bloch_solve(kap, g["factors"], n0=n0, L=L, ieigs=ie, m=m, method=1,
                                                max_nested=40, max_steps=80, tol=float(g["tol"]), relative=0,
                                                extrapolation="n", wave=1)
    assert st == 0 and res[:, :ie].max() <= float(g["tol"])
    assert np.abs(lam[:, :ie] - g["lam"][:, :ie]).max() < 2e-6
