"""Generate the golden vectors of the eigensolver path from the reference.

Runs the reference's own modules (compiled unmodified by
``make -C oracle ref`` into oracle/_ref/libmaxwell_ref.so) on seeded inputs
and writes ``tests/golden/*.npz``.  Needs the reference sources at build
time; the fixtures it writes are committed so that the tests run anywhere.

    OPENBLAS_NUM_THREADS=1 python tests/golden/gen_golden.py            # all fixtures
    OPENBLAS_NUM_THREADS=1 python tests/golden/gen_golden.py hiptmair   # hiptmair_n16.npz only
"""
from __future__ import annotations

import os
import sys

os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from oracle import RefLib, build_oracle  # noqa: E402


def cvec(rng, n):
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


def seam_consistent(rng, n):
    """Random kappa in [1/12, 1] whose last row equals the row below it and
    whose last column is constant, so that the reference's matrix-free
    operator (which reads those cells with a shifted index) is exact."""
    k = 1.0 / (1.0 + 11.0 * rng.random((n, n)))
    k[-1, :] = k[-2, :]
    k[:, -1] = k[0, -1]
    return k.reshape(-1)


def gen_ops(R: RefLib, n: int, seed: int) -> dict:
    rng = np.random.default_rng(seed)
    out = {"n": n}
    xf, yf = np.exp(0.7j), np.exp(-1.3j)
    out["xf"], out["yf"] = xf, yf
    kap_s = seam_consistent(rng, n)
    kap_g = 1.0 / (1.0 + 11.0 * rng.random(n * n))
    x, y, b = cvec(rng, 2 * n * n), cvec(rng, 2 * n * n), cvec(rng, 2 * n * n)
    v, w = cvec(rng, n * n), cvec(rng, n * n)
    out.update(kappa_seam=kap_s, kappa_gen=kap_g, x=x, y=y, b=b, v=v, w=w)
    alpha, beta = 1.3, 0.7
    out["alpha"], out["beta"] = alpha, beta
    out["addeval"] = R.addeval_edge(n, kap_s, xf, yf, alpha, beta, x, y)
    out["products"] = R.products_edge(n, kap_s, xf, yf, 1.0, 1.0, x, y)
    out["dense_edge"] = R.dense_edge(n, kap_g, xf, yf, 1.0, 1.0) if n <= 8 else np.zeros(0)
    for d, name in ((0, "fwd"), (1, "bwd"), (2, "symm")):
        out[f"gs_{name}"] = R.gs_edge(n, kap_g, xf, yf, 1.0, 1.0, d, b, x)
        out[f"ngs_{name}"] = R.gs_node(n, xf, yf, 1.0, d, v, w)
    nc = n // 2
    c = cvec(rng, 2 * nc * nc)
    vc = cvec(rng, nc * nc)
    out.update(c=c, vc=vc)
    out["prolong"] = R.transfer_edge(nc, xf, yf, 1.0, 0, c, x)
    out["restrict"] = R.transfer_edge(nc, xf, yf, 1.0, 1, x, c)
    out["nprolong"] = R.transfer_node(nc, xf, yf, 1.0, 0, vc, v)
    out["nrestrict"] = R.transfer_node(nc, xf, yf, 1.0, 1, v, vc)
    out["naddeval"] = R.addeval_node(n, xf, yf, 0.9, v, w)
    out["gradient"] = R.gradient(n, xf, yf, 1.0, 0, v, x)
    out["adjgradient"] = R.gradient(n, xf, yf, 1.0, 1, x, v)
    out["center"] = R.center_edge(n, x)
    if n <= 8:
        out["dense_node_gamma"] = R.dense_node(n, 1.0, 1.0, 1)
        out["dense_node_k"] = R.dense_node(n, xf, yf, 1)
    out["coarsen"] = R.coarsen_kappa(n // 4, 2, kap_g)
    return out


def quadrant_kappa(rng, n):
    """Random kappa in the lower-left quadrant, 1 elsewhere: seam-consistent
    (see seam_consistent) on every level of the coarsening hierarchy."""
    k = np.ones((n, n))
    k[: n // 2, : n // 2] = 1.0 / (1.0 + 11.0 * rng.random((n // 2, n // 2)))
    return k.reshape(-1)


def gen_vcycle(R: RefLib, seed: int) -> dict:
    rng = np.random.default_rng(seed)
    n0, L = 4, 2
    n = n0 << L
    kap = quadrant_kappa(rng, n)
    xf, yf = np.exp(0.4j), np.exp(2.1j)
    b = cvec(rng, 2 * n * n)
    bn = cvec(rng, n * n)
    out = dict(n0=n0, L=L, kappa=kap, xf=xf, yf=yf, b=b, bn=bn)
    out["vcycle_edge"] = R.vcycle_edge(n0, L, kap, xf, yf, 2, 1, 2, b, np.zeros_like(b))
    out["vcycle_edge_nocoarse"] = R.vcycle_edge(n0, L, kap, xf, yf, 2, 0, 1, b, np.zeros_like(b))
    out["vcycle_node"] = R.vcycle_node(n0, L, xf, yf, 2, 1, 3, bn, np.zeros_like(bn))
    out["vcycle_node_gamma"] = R.vcycle_node(n0, L, 1.0, 1.0, 2, 1, 3, bn, np.zeros_like(bn))
    e = cvec(rng, 2 * n * n)
    out["e"] = e
    out["pinvit"] = R.pinvit(n0, L, kap, xf, yf, 2, 2, 5, 40.0, e)
    return out


DISC_C1 = [[8.9, 0.5, 0.5, 0.2]]


def disc_kappa(n, discs, eps_base=1.0):
    """setpattern_grid2d's rule (lower-left corner of each cell)."""
    h = 1.0 / n
    k = np.full(n * n, 1.0 / eps_base)
    for j in range(n):
        for i in range(n):
            for e, cx, cy, r in discs:
                if (i * h - cx) ** 2 + (j * h - cy) ** 2 <= r * r:
                    k[i + j * n] = 1.0 / e
    return k


def gen_eigs(R: RefLib) -> dict:
    n0, L = 8, 2
    n = n0 << L
    kap = disc_kappa(n, DISC_C1)
    ks = [(0.0, 0.0), (np.pi / 2, 0.0), (np.pi, 0.0), (np.pi, np.pi / 2), (np.pi, np.pi),
          (np.pi / 2, np.pi / 2)]
    fac = np.array([[np.exp(1j * a), np.exp(1j * b)] for a, b in ks])
    st, lam, steps, dfc = R.bloch_solve(kap, fac, n0=n0, L=L, ieigs=8, throwaway=4,
                                        pinvit_steps=80, bloch_steps=80, tol=1e-9,
                                        extrapolation="2", nthreads=1)
    assert st == 0
    return dict(n0=n0, L=L, kappa=kap, kpoints=np.array(ks), factors=fac, ieigs=8, m=12,
                lam=lam, steps=steps, defects=dfc, tol=1e-9)


def gen_hiptmair(R: RefLib, seed: int) -> dict:
    """The point smoother (gs*_simple_edge2d) and the Hiptmair cycle
    (hcycle_edge2d) on a 16^2 grid with a random kappa in one quadrant,
    equal across the seams on every level (so that the reference's
    matrix-free residuals use the kappa its dense matrix does)."""
    rng = np.random.default_rng(seed)
    n0, L = 4, 2
    n = n0 << L
    kap = quadrant_kappa(rng, n)
    xf, yf = np.exp(0.9j), np.exp(-0.6j)
    b, x = cvec(rng, 2 * n * n), cvec(rng, 2 * n * n)
    out = dict(n0=n0, L=L, kappa=kap, xf=xf, yf=yf, b=b, x=x)
    for d, name in ((0, "fwd"), (1, "bwd"), (2, "symm")):
        out[f"simple_{name}"] = R.gs_edge_simple(n, kap, xf, yf, 1.0, 1.0, d, b, x)
    out["hcycle"] = R.hcycle_edge(n0, L, kap, xf, yf, 2, 1, 2, b, np.zeros_like(b))
    out["hcycle_nocoarse"] = R.hcycle_edge(n0, L, kap, xf, yf, 2, 0, 1, b, np.zeros_like(b))
    return out


def main() -> None:
    build_oracle(ref=True)
    R = RefLib()
    if sys.argv[1:] == ["hiptmair"]:
        np.savez_compressed(os.path.join(HERE, "hiptmair_n16.npz"), **gen_hiptmair(R, 21))
        return
    np.savez_compressed(os.path.join(HERE, "ops_n8.npz"), **gen_ops(R, 8, 8))
    np.savez_compressed(os.path.join(HERE, "ops_n16.npz"), **gen_ops(R, 16, 16))
    np.savez_compressed(os.path.join(HERE, "vcycle_n16.npz"), **gen_vcycle(R, 3))
    np.savez_compressed(os.path.join(HERE, "eigs_n32_disc.npz"), **gen_eigs(R))
    np.savez_compressed(os.path.join(HERE, "hiptmair_n16.npz"), **gen_hiptmair(R, 21))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
