"""The launch-shape autotuner (mxg_autotune): it picks, per tunable, one of
its candidates, keeps the choice for the process, and a solve under the chosen
shapes still matches the reference's eigenvalues (the shapes change only the
launch geometry and the order of floating-point sums)."""
import numpy as np
import pytest

import maxwell_gb300 as mx

pytestmark = pytest.mark.gpu


def _solve(g):
    ie, m = int(g["ieigs"]), int(g["m"])
    s = mx.Solver(g["kappa"], n0=int(g["n0"]), L=int(g["L"]), ieigs=ie, m=m, method=1, precision=1,
                  max_nested=40, max_steps=40, wave=len(g["factors"]), relative=0, tol=float(g["tol"]))
    lam, steps, res = s.solve(g["factors"])
    return lam[:, :ie], res[:, :ie]


def test_autotune_choice_and_solve(golden):
    g = golden("eigs_n32_disc.npz")
    default = mx.get_tuning()
    try:
        t = mx.autotune(256, 8, 8, reps=3)
        assert t["gram_waves"] in (1, 2, 4, 8, 16)
        assert t["combine_ctas"] in (1, 2, 3, 4)
        assert t["residual_sites"] in (8, 16, 32, 64, 128)
        assert t["node_strip"] in (0, 64, 128) and t["node_band"] in (4, 8, 16, 32, 64)
        assert t["restrict_strip_log2"] == default["restrict_strip_log2"]   # not searched
        assert mx.get_tuning() == t
        # the extreme shapes too (strips of coarse rows at every level, and at none)
        for shape in ({"gram_waves": 1, "combine_ctas": 1, "residual_sites": 128, "node_strip": 64, "node_band": 1,
                       "restrict_strip_log2": 0},
                      {"gram_waves": 16, "combine_ctas": 4, "residual_sites": 8, "node_strip": 128,
                       "node_band": 64, "restrict_strip_log2": 62}, t):
            mx.set_tuning(**shape)
            lam, res = _solve(g)
            want = g["lam"][:, :int(g["ieigs"])]
            assert np.abs(lam - want).max() / want.max() < 1e-8, shape
            assert res.max() <= float(g["tol"])
    finally:
        mx.set_tuning(**default)
