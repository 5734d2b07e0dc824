"""Golden eigenvalues at two of the task's configurations.

* ``headline_n512_disc.npz`` -- the 512^2 benchmark configuration (disc
  eps = 12 of radius 0.3 centred in the unit cell, 12 wanted pairs with
  block 16, LOBPCG, 7 levels 512 .. 8) at Gamma, X, M and one interior point
  of the benchmark's Gamma-X-M-Gamma path, solved by the oracle restatement
  (oracle/maxwell_oracle.c, complex128 throughout) to a relative residual of
  1e-10, i.e. with eigenvalues far more accurate than the 1e-8 the GPU solver
  is held to.
* ``config1_n64_disc.npz`` -- the CPU-runnable configuration (64^2, disc
  eps = 8.9 of radius 0.2, 16 k-points spaced evenly in arc length along
  Gamma-X-M-Gamma, 10 wanted pairs with block 12, block PINVIT, 4 levels
  64 .. 8) solved by the reference's own modules (oracle/_ref, compiled
  unmodified by ``make -C oracle ref``) following exp_bloch2d's flow: coarse
  eigenproblem, nested iteration, then the Bloch scan with second-order
  Rayleigh-Ritz extrapolation, block PINVIT to the absolute defect 1e-8.

Permittivities follow setpattern_grid2d's rule (grid2d.c:171-218); the
fixtures store the geometry, the number of cells inside the disc and the
sum of 1/eps, not the arrays.

    python tests/golden/gen_headline.py [headline|config1]
"""
from __future__ import annotations

import os
import sys
import time

os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from oracle import Oracle, RefLib, build_oracle  # noqa: E402


def path_points(nk: int) -> np.ndarray:
    """nk points evenly spaced in arc length along Gamma-X-M-Gamma."""
    seg = [np.pi, np.pi, np.pi * np.sqrt(2.0)]
    pts = []
    for t in np.linspace(0.0, sum(seg), nk):
        if t <= seg[0]:
            pts.append((t, 0.0))
        elif t <= seg[0] + seg[1]:
            pts.append((np.pi, t - seg[0]))
        else:
            s = (t - seg[0] - seg[1]) / np.sqrt(2.0)
            pts.append((np.pi - s, np.pi - s))
    return np.array(pts)


def headline(O: Oracle) -> None:
    n0, L, ieigs, m, tol = 8, 6, 12, 16, 1e-10
    n = n0 << L
    disc = np.array([12.0, 0.5, 0.5, 0.3])
    kap = O.disc_kappa(n, [disc], 1.0)
    kpts = np.array([(0.0, 0.0), (np.pi, 0.0), (np.pi, np.pi), tuple(path_points(32)[10])])
    fac = np.exp(1j * kpts)
    lam, res, steps = [], [], []
    for q in range(len(kpts)):
        t0 = time.time()
        st, l, s, r, _ = O.bloch_solve(kap, fac[q:q + 1], n0=n0, L=L, ieigs=ieigs, m=m, method=1, max_nested=5,
                                       max_steps=100, tol=tol, relative=1, extrapolation="n", wave=1)
        assert st == 0
        print(f"k-point {q}: {s[0]} steps, max residual {r[0, :ieigs].max():.2e}, {time.time() - t0:.0f} s",
              flush=True)
        lam.append(l[0]); res.append(r[0]); steps.append(s[0])
    np.savez(os.path.join(HERE, "headline_n512_disc.npz"), n0=n0, L=L, ieigs=ieigs, m=m, tol=tol, disc=disc,
             eps_base=1.0, inside=int((kap < 1.0).sum()), kappa_sum=float(kap.sum()), kpoints=kpts, factors=fac,
             lam=np.array(lam), res=np.array(res), steps=np.array(steps))


def config1(O: Oracle) -> None:
    build_oracle(ref=True)
    R = RefLib()
    n0, L, ieigs, throwaway, tol = 8, 3, 10, 2, 1e-8
    n = n0 << L
    disc = np.array([8.9, 0.5, 0.5, 0.2])
    kap = O.disc_kappa(n, [disc], 1.0)
    kpts = path_points(16)
    fac = np.exp(1j * kpts)
    t0 = time.time()
    st, lam, steps, dfc = R.bloch_solve(kap, fac, n0=n0, L=L, ieigs=ieigs, throwaway=throwaway, pinvit_steps=200,
                                        bloch_steps=400, tol=tol, extrapolation="2", nthreads=8)
    assert st == 0
    print(f"config 1: steps {steps.tolist()}, max defect {dfc[:, :ieigs].max():.2e}, {time.time() - t0:.0f} s")
    np.savez(os.path.join(HERE, "config1_n64_disc.npz"), n0=n0, L=L, ieigs=ieigs, m=ieigs + throwaway, tol=tol,
             disc=disc, eps_base=1.0, inside=int((kap < 1.0).sum()), kappa_sum=float(kap.sum()), kpoints=kpts,
             factors=fac, lam=lam, defects=dfc, steps=steps)


if __name__ == "__main__":
    build_oracle()
    O = Oracle()
    O.set_threads(os.cpu_count() or 1)
    which = sys.argv[1:] or ["config1", "headline"]
    if "config1" in which:
        config1(O)
    if "headline" in which:
        headline(O)
