"""The drop-in boundary used the way the reference uses its own modules: a C
program (tests/c_driver_pinvit.c) that drives only the mirror API --
setpattern_grid2d, the coarse dense eigenproblem (densematrix_edge2d +
sygv_matrix), prolongation_edge2d, pinvit_edge2d, the block Gram
(energyprod/massprod of all pairs) + sygv_matrix + the Ritz combination --
in the order of exp_bloch2d.c:335-1018, compiled with gcc against
include/maxwell_gb300.h and linked with the library.  Its eigenvalues for
five k-points of a 32^2 disc agree with the reference's own solve of the same
problem (tests/golden/eigs_n32_disc.npz, absolute defect 1e-9) to 1e-8."""
import os
import subprocess

import numpy as np
import pytest

import maxwell_gb300 as mx

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    lib = mx.LIB_PATH
    exe = str(tmp_path_factory.mktemp("cdriver") / "c_driver_pinvit")
    r = subprocess.run(["gcc", "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror",
                        os.path.join(ROOT, "tests", "c_driver_pinvit.c"), "-I", os.path.join(ROOT, "include"),
                        "-o", exe, "-L", os.path.dirname(lib), "-l:" + os.path.basename(lib),
                        "-Wl,-rpath," + os.path.dirname(lib), "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_driver_matches_reference(driver, golden):
    g = golden("eigs_n32_disc.npz")
    ie, m = int(g["ieigs"]), int(g["m"])
    ks = g["kpoints"][1:]                                   # the five k-points away from Gamma
    args = [str(int(g["n0"])), str(int(g["L"])), str(ie), str(m), "1e-9", "400", "8.9", "0.2"]
    args += [f"{v:.17g}" for kp in ks for v in kp]
    r = subprocess.run([driver] + args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rows = [list(map(float, line.split())) for line in r.stdout.strip().splitlines()]
    assert len(rows) == len(ks)
    lam = np.array([row[1:] for row in rows])
    want = g["lam"][1:, :ie]
    assert (np.abs(lam - want) / want).max() < 1e-8, (lam, want)
