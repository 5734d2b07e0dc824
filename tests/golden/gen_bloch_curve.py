"""Golden eigenvalues along the reference's own Bloch curve, from its driver
program.

Builds the reference's exp_bloch2d (``make -C oracle ref-driver``: the driver
and its modules compiled unmodified, NetCDF and picture output replaced by
no-ops), runs it non-interactively through its ``maxwell_*`` environment
variables on a 16^2 grid with the driver's Kivshar pattern (one disc,
eps = 11.56, r = 0.18) and 4 Bloch steps per edge of the Gamma-X-M-Gamma
curve, and writes the eigenvalues of its protocol file to
``tests/golden/bloch_curve_n16_kivshar.npz``.  The run happens under
oracle/_ref (not committed); only the fixture is.

    python tests/golden/gen_bloch_curve.py
"""
from __future__ import annotations

import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
RUN = os.path.join(ROOT, "oracle", "_ref", "curve_run")
EXE = os.path.join(ROOT, "oracle", "_ref", "exp_bloch2d")

N0, LEVELS, IEIGS, THROWAWAY, STEPS_PER_EDGE, TOL = 8, 1, 4, 4, 4, 1e-8
DISC = (11.56, 0.5, 0.5, 0.18)   # the driver's Kivshar pattern (exp_bloch2d.c:64-76)

SETTINGS = dict(
    maxwell_coarse=N0, maxwell_levels=LEVELS, maxwell_permittivity="k", maxwell_eigs=IEIGS,
    maxwell_throwaway=THROWAWAY, maxwell_chern=IEIGS, maxwell_continuity="s",
    maxwell_blochsteps=STEPS_PER_EDGE, maxwell_extra="2", maxwell_protocol="bloch2d.dat",
    maxwell_grid="grid.png", maxwell_cdf="bloch2d.nc", maxwell_stop="r", maxwell_residual=TOL,
    maxwell_pinvit=40, maxwell_bloch=80, maxwell_visual="n")


def curve_point(pt: int, steps: int) -> tuple[float, float]:
    """The driver's Bloch curve (exp_bloch2d.c:22-47)."""
    if pt < steps:
        return math.pi * pt / steps, 0.0
    if pt < 2 * steps:
        return math.pi, math.pi * (pt - steps) / steps
    t = math.pi * (1.0 - (pt - 2 * steps) / (1.41 * steps))
    return t, t


def main() -> None:
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref-driver"], check=True)
    os.makedirs(RUN, exist_ok=True)
    env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1",
               **{k: str(v) for k, v in SETTINGS.items()})
    with open(os.path.join(RUN, "run.log"), "w") as log:
        subprocess.run([EXE], cwd=RUN, env=env, stdin=subprocess.DEVNULL, stdout=log, stderr=log, check=True)
    eigs = IEIGS + THROWAWAY
    lam, iters, chern = [], [], []
    with open(os.path.join(RUN, "bloch2d.dat")) as f:
        protocol = f.read().splitlines()
    header = [line for line in protocol if line.startswith("#")]
    if True:
        for line in protocol:
            if line.startswith("#") or not line.strip():
                continue
            v = line.split()
            lam.append([float(x) for x in v[1:1 + eigs]])
            if len(v) > 1 + eigs:
                iters.append(int(v[1 + eigs]))
                c = [float(x) for x in v[4 + eigs:4 + eigs + 2 * IEIGS]]
                chern.append([complex(c[2 * i], c[2 * i + 1]) for i in range(IEIGS)])
            else:   # the starting point: eigenvalues only
                iters.append(0)
                chern.append([0j] * IEIGS)
    npts = int(3.41 * STEPS_PER_EDGE + 1)
    assert len(lam) == npts, (len(lam), npts)
    ks = np.array([curve_point(p, STEPS_PER_EDGE) for p in range(npts)])
    fac = np.exp(1j * ks)
    np.savez_compressed(os.path.join(HERE, "bloch_curve_n16_kivshar.npz"),
                        n0=N0, L=LEVELS, disc=np.array(DISC), eps_base=1.0, ieigs=IEIGS, m=IEIGS + THROWAWAY,
                        tol=TOL, kpoints=ks, factors=fac, lam=np.array(lam), iterations=np.array(iters),
                        chern=np.array(chern), protocol_header=np.array(header))
    print("points", npts, "lam", np.array(lam).shape)


if __name__ == "__main__":
    main()
