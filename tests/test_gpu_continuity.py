"""Eigenvector continuity and Chern partial sums (mxg_bloch_continuity,
exp_bloch2d.c:1058-1216) against the oracle's literal restatement of the
reference's code applied to the same eigenvectors: the k-points of the
reference driver's own curve (Kivshar disc, 16^2, 14 points with corners at
points 0, 4, 8 and 13), solved by the GPU in one wave; the raw eigenvectors
go to the oracle, the GPU adjusts its own.  Swap counts and the reordered
eigenvalues agree exactly, the Chern partial sums to 1e-9, the adjusted
eigenvectors to 1e-9 up to a unit factor each, and the GPU's adjusted
vectors make every overlap with their guess real and non-negative."""
import numpy as np
import pytest

import maxwell_gb300 as mx

pytestmark = pytest.mark.gpu


def curve_vertices(nk, steps_per_edge):
    """blochcurve's corner flags (exp_bloch2d.c:45-46), with the first point
    a corner as the scan starts (exp_bloch2d.c:447)."""
    return np.array([1 if p in (0, steps_per_edge, 2 * steps_per_edge, nk - 1) else 0 for p in range(nk)],
                    np.int32)


@pytest.mark.parametrize("continuity", ["n", "s", "r"])
def test_continuity_matches_oracle(oracle, golden, continuity):
    g = golden("bloch_curve_n16_kivshar.npz")
    n0, L, ie, m = int(g["n0"]), int(g["L"]), int(g["ieigs"]), int(g["m"])
    n = n0 << L
    kap = oracle.disc_kappa(n, [g["disc"]], float(g["eps_base"]))
    fac = g["factors"]
    nk = len(fac)
    s = mx.Solver(kap, n0=n0, L=L, ieigs=ie, m=m, method=1, precision=1, wave=nk, relative=0, tol=1e-9,
                  max_nested=40, max_steps=80)
    lam, steps, res = s.solve(fac)
    assert res[:, :ie].max() <= 1e-9
    raw = s.eigenvectors()
    vertex = curve_vertices(nk, 4)
    lam_g, chern_g, sign_g = s.continuity(lam, vertex, continuity, chern_vectors=ie)
    adj = s.eigenvectors()
    v_o, lam_o, chern_o, sign_o = oracle.continuity(n, fac, ie, vertex, continuity, ie, raw, lam)
    assert np.array_equal(sign_g, sign_o)
    assert np.array_equal(lam_g, lam_o)
    assert np.abs(chern_g - chern_o).max() < 1e-9
    # The adjusted vectors: where a vector changes band between neighbouring
    # points (the block's unconverged vectors, and with 's' crossing wanted
    # ones), its overlap with the previous point's vector -- whose phase the
    # adjustment takes -- is rounding noise on both sides, and the phase
    # difference travels down the chain (the Chern sums, made of relative
    # phases, do not see it).  So every adjusted vector equals the oracle's
    # up to one unit factor, and the GPU's own vectors meet the rule itself:
    # e_i^H M guess_i real and non-negative, guess_i the previous point's
    # vector (or 2 e_i(l-1) - e_i(l-2) away from corners), wherever that
    # overlap is not rounding noise
    scale = np.abs(v_o).max()
    for l in range(nk):
        for i in range(m):
            z = np.vdot(v_o[l, i], adj[l, i])
            ph = z / abs(z)
            assert np.abs(adj[l, i] - ph * v_o[l, i]).max() < 1e-9 * scale, (l, i)
    if continuity != "n":
        for l in range(1, nk):
            for i in range(m):
                prev2 = adj[l - 2, i] if l > 1 else np.zeros_like(adj[0, i])
                guess = adj[l - 1, i] if vertex[l - 1] else 2 * adj[l - 1, i] - prev2
                p = oracle.massprod_edge(n, *fac[l], guess, adj[l, i])
                if abs(p) > 1e-6:   # else a band change: the overlap, and the phase, is noise
                    assert abs(p.imag) <= 1e-9 * abs(p) and p.real >= 0, (l, i, p)
    if continuity == "n":
        assert np.array_equal(adj, raw)
