"""Golden eigenvalues on the reference's own full-zone grid, from its surface
driver program.

Builds the reference's exp_blochsurf (``make -C oracle ref-surf``: the driver
and its modules compiled unmodified, picture output replaced by no-ops),
runs it non-interactively through its ``maxwell_*`` environment variables on
a 16^2 grid with the driver's Kivshar pattern (one disc, eps = 11.56,
r = 0.18) and 4 Bloch steps per edge (k = 2 pi i / 3 - pi: no Gamma on the
grid), absolute residual 1e-8, and writes the eigenvalues of its protocol
file to ``tests/golden/blochsurf_n16_kivshar.npz``.  The run happens under
oracle/_ref (not committed); only the fixture is.

    python tests/golden/gen_blochsurf.py
"""
from __future__ import annotations

import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
RUN = os.path.join(ROOT, "oracle", "_ref", "surf_run")
EXE = os.path.join(ROOT, "oracle", "_ref", "exp_blochsurf")

N0, LEVELS, IEIGS, THROWAWAY, STEPS, TOL = 8, 1, 4, 4, 4, 1e-8
DISC = (11.56, 0.5, 0.5, 0.18)   # the driver's Kivshar pattern

SETTINGS = dict(
    maxwell_coarse=N0, maxwell_levels=LEVELS, maxwell_permittivity="k", maxwell_eigs=IEIGS,
    maxwell_throwaway=THROWAWAY, maxwell_blochsteps=STEPS, maxwell_protocol="blochsurf.dat",
    maxwell_grid="grid.png", maxwell_pinvit=40, maxwell_bloch=80, maxwell_residual=TOL)


def main() -> None:
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref-surf"], check=True)
    os.makedirs(RUN, exist_ok=True)
    env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1",
               **{k: str(v) for k, v in SETTINGS.items()})
    with open(os.path.join(RUN, "run.log"), "w") as log:
        subprocess.run([EXE], cwd=RUN, env=env, stdin=subprocess.DEVNULL, stdout=log, stderr=log, check=True)
    eigs = IEIGS + THROWAWAY
    with open(os.path.join(RUN, "blochsurf.dat")) as f:
        protocol = f.read().splitlines()
    header = [line for line in protocol if line.startswith("#")]
    index, lam, iters = [], [], []
    for line in protocol:
        if line.startswith("#") or not line.strip():
            continue
        v = line.split()
        index.append((int(v[0]), int(v[1])))
        lam.append([float(x) for x in v[2:2 + eigs]])
        iters.append(int(v[2 + eigs]))
    assert sorted(index) == sorted((ix, iy) for ix in range(STEPS) for iy in range(STEPS)), index
    ks = 2.0 * math.pi * np.arange(STEPS) / (STEPS - 1) - math.pi   # exp_blochsurf.c:25-36
    fac = np.array([[np.exp(1j * ks[ix]), np.exp(1j * ks[iy])] for ix, iy in index])
    np.savez_compressed(os.path.join(HERE, "blochsurf_n16_kivshar.npz"),
                        n0=N0, L=LEVELS, disc=np.array(DISC), eps_base=1.0, ieigs=IEIGS, m=eigs, tol=TOL,
                        steps=STEPS, index=np.array(index), factors=fac, lam=np.array(lam),
                        iterations=np.array(iters), protocol_header=np.array(header))
    print("points", len(index), "lam", np.array(lam).shape)


if __name__ == "__main__":
    main()
