"""Benchmark: k-points/s of the Bloch eigensolver at 512^2, 12 eigenpairs to a
relative residual of 1e-8 (mixed precision, batched over k-points) next to
the plain FP64 GPU solver and the CPU oracle.

Workload (one "step" = one complete solve of the batch): the unit cell
meshed as 512 x 512 cells, eps = 12 inside the centred disc of radius 0.3,
eps = 1 outside; 32 Bloch k-points spaced evenly in arc length along
Gamma-X-M-Gamma; 12 wanted pairs with block 16 via LOBPCG; 7 multigrid levels
(512 .. 8) in FP32 complex; eigenvector block, residuals, Rayleigh quotients
and the eigenvector-eigenvector Gram entries in float-float arithmetic, the
Gram entries that involve a search direction in FP32 (the residual form for
the eigenvector-search-direction ones), Cholesky-QR and the Ritz
eigenproblem in FP64; stopping rule relative residual <= 1e-8 for every
wanted pair.  Every step solves the 32 k-points from scratch (coarse
eigenproblem, nested iteration, LOBPCG), so no step can reuse another's
results.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank selects the GPU of its LOCAL_RANK and solves its own
32 k-points (rank r takes every N-th point of a 32*N-point path): per-GPU
work is fixed, no data-path collective.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N0, LEVELS = 8, 6            # 8 << 6 = 512
EPS_DISC, R_DISC = 12.0, 0.3
NK = 32
IEIGS, BLOCK = 12, 16
TOL = 1e-8
METRIC = "k-points/s at 512^2 grid, 12 eigenpairs @1e-8 residual: mixed+batched vs FP64"


def gamma_x_m_gamma(nk: int) -> np.ndarray:
    """nk points evenly spaced in arc length along Gamma-X-M-Gamma, both ends
    at Gamma (kx, ky in units where the zone edge is pi)."""
    seg = [np.pi, np.pi, np.pi * np.sqrt(2.0)]
    total = sum(seg)
    pts = []
    for t in np.linspace(0.0, total, nk):
        if t <= seg[0]:
            pts.append((t, 0.0))
        elif t <= seg[0] + seg[1]:
            pts.append((np.pi, t - seg[0]))
        else:
            s = (t - seg[0] - seg[1]) / np.sqrt(2.0)
            pts.append((np.pi - s, np.pi - s))
    return np.array(pts)


def disc_kappa(n: int) -> np.ndarray:
    """1/eps per cell by setpattern_grid2d's rule (lower-left corner inside the disc)."""
    h = 1.0 / n
    i = np.arange(n)
    X, Y = np.meshgrid(i * h, i * h)   # X varies along columns (i), Y along rows (j)
    inside = (X - 0.5) ** 2 + (Y - 0.5) ** 2 <= R_DISC ** 2
    k = np.where(inside, 1.0 / EPS_DISC, 1.0)
    return np.ascontiguousarray(k.reshape(-1))


def factors_of(kpts: np.ndarray) -> np.ndarray:
    return np.stack([np.exp(1j * kpts[:, 0]), np.exp(1j * kpts[:, 1])], axis=1)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def rank_device() -> int:
    """The GPU of this process: one process per GPU, the GPU of its
    LOCAL_RANK (0 without torchrun)."""
    return int(os.environ.get("LOCAL_RANK", "0"))


def rank_kpoints(ws: int, rank: int) -> np.ndarray:
    """The k-points of one rank: every ws-th point of a 32*ws-point path, so
    each rank solves NK independent k-points (weak scaling) and the ranks
    together cover the path once."""
    return gamma_x_m_gamma(NK * ws)[rank::ws]


def max_over_ranks(values):
    """Element-wise maximum of per-rank timings (no-op on one process)."""
    if int(os.environ.get("WORLD_SIZE", "1")) == 1:
        return [float(v) for v in values]
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(rank_device()),
                                          f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.samples.append(parts)

    def stop(self) -> dict:
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["not sampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for s in self.samples for q in range(4) if s[3 + q].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def _oracle(threads: int):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    O = Oracle()
    O.set_threads(threads)
    return O


# nested iteration on the coarser levels: the reference's default residual
# rule, at most 20 block steps per level until the wanted pairs' defect is
# below 1e-2 (exp_bloch2d.c:296-321 stopping 'r', 628)
MAX_NESTED, NESTED_TOL = 20, 1e-2
# the reference driver's flow for a sequence of k-points (exp_bloch2d.c:781-1053):
# one k-point after the other, each started by second-order Rayleigh-Ritz
# extrapolation from the two before it (its default, exp_bloch2d.c:283)
CPU_KW = dict(n0=N0, L=LEVELS, ieigs=IEIGS, m=BLOCK, method=1, max_nested=MAX_NESTED, nested_tol=NESTED_TOL,
              max_steps=60, relative=1,
              tol=TOL, extrapolation="2", wave=1)


def cpu_path_solve(threads: int, kap, fac):
    """The oracle port (oracle/maxwell_oracle.c, OpenMP on `threads` host
    threads) over consecutive k-points of the path, the first from a cold
    start and every later one warm-started from the ones before it; returns
    eigenvalues, block steps, residuals and seconds per k-point."""
    O = _oracle(threads)
    st, lam, steps, res, _, secs = O.bloch_solve(kap, fac, want_times=True, **CPU_KW)
    if st != 0:
        raise RuntimeError(f"oracle solve failed with status {st}")
    return lam, steps, res, secs


def cpu_baseline(kap, fac, threads: int, lam_gpu) -> dict:
    """A bounded sample of the same workload on the host cores: the first
    three k-points of the path solved to the relative residual 1e-8 -- Gamma
    and the point after it from cold starts (the Gamma block lacks the two
    lowest bands of k != 0, so the port starts the next point cold), the
    third warm-started.  The rate of the whole 32-point path is those two
    cold k-points plus 30 warm ones at the sampled warm time; only the
    number of k-points is extrapolated.  The sample's eigenvalues are also
    the CPU FP64 check of the GPU's at the same k-points."""
    nks = 3
    lam, steps, res, secs = cpu_path_solve(threads, kap, fac[:nks])
    t_cold, t_warm = float(secs[0] + secs[1]), float(np.mean(secs[2:]))
    per_path = t_cold + (NK - 2) * t_warm
    diff = np.abs(lam_gpu[:nks, :IEIGS] - lam[:, :IEIGS]) / np.abs(lam[:, :IEIGS])
    return {"value": NK / per_path, "unit": "k-points/s", "cores": threads, "kind": "port",
            "sample": (f"the first {nks} k-points of the 512^2 path solved to relative residual 1e-8 by the "
                       f"oracle port: cold starts at Gamma and the next point {secs[0]:.1f}, {secs[1]:.1f} s "
                       f"({int(steps[0])}, {int(steps[1])} LOBPCG steps after the nested iteration), warm start "
                       f"{', '.join(f'{t:.1f}' for t in secs[2:])} s "
                       f"({', '.join(str(int(q)) for q in steps[2:])} steps); 32-point path = 2 cold + 30 warm"),
            "measured_seconds": [float(t) for t in secs], "steps": [int(q) for q in steps],
            "max_rel_eig_diff_gpu_vs_cpu": float(diff.max()),
            "max_rel_residual_cpu": float(res[:, :IEIGS].max())}


def fp64_residual_check(mx, n, kap, fac, lam, vec) -> float:
    """Largest relative residual ||(A+M)e - mu M e|| / (mu ||M e||) of the
    wanted pairs, recomputed from the returned eigenvectors with the
    library's complex128 operator kernels (addeval_edge2d_gpu) and norms."""
    K, m = vec.shape[0], vec.shape[1]
    g = mx.Grid(n, K, kap, fac)
    e = mx.Edge(g, m, mx.C128, vec)
    r, v = mx.Edge(g, m, mx.C128), mx.Edge(g, m, mx.C128)
    mu = lam + 1.0
    shift = np.ascontiguousarray(1.0 - mu)
    mx.check(mx.lib().addeval_shifted_edge2d_gpu(1.0, mx._ptr(shift), e.h, r.h))
    mx.check(mx.lib().addeval_edge2d_gpu(mx.fz(0.0), mx.fz(1.0), e.h, v.h))
    nr, nv = np.zeros(K * m), np.zeros(K * m)
    mx.check(mx.lib().norm2_edge2d_gpu(r.h, mx._ptr(nr)))
    mx.check(mx.lib().norm2_edge2d_gpu(v.h, mx._ptr(nv)))
    rel = (nr / (np.abs(mu).reshape(-1) * nv)).reshape(K, m)
    return float(rel[:, :IEIGS].max())


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per timed
# sequence at 32 k-points, scaled by 8 from ncu captures at 4 k-points (the
# full 32-k workload holds > 30 GB on the device): node GS sweep
# (profiles/node_gs_512x512_k4_ncu.md), AFW sweep
# (profiles/afw_rowpair_512x512_k4_ncu.md), Gram
# (profiles/block_gram_split_512x512_k4_ncu.md)
TRAFFIC_32K = {"node_gs": 8 * 484.0e6, "afw": 8 * 2 * 648.1e6, "gram": 8 * 3.501e9}


def run_ours(args):
    import maxwell_gb300 as mx
    ws, rank = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if not mx.lib().mxg_device_ok():
        raise RuntimeError("no CUDA device")
    dev = rank_device()
    mx.check(mx.lib().mxg_set_device(dev), "mxg_set_device")
    n = N0 << LEVELS
    kap = disc_kappa(n)
    kpts = rank_kpoints(ws, rank)
    fac = factors_of(kpts)

    def make(precision, wave):
        return mx.Solver(kap, n0=N0, L=LEVELS, ieigs=IEIGS, m=BLOCK, method=1, precision=precision,
                         max_nested=MAX_NESTED, nested_tol=NESTED_TOL, max_steps=60, wave=wave, relative=1,
                         tol=TOL)

    if args.autotune:
        mx.autotune(n, NK, BLOCK, 3)
    s = make(1, NK)
    for _ in range(args.warmup):
        s.solve(fac)
    clocks = Clocks()
    clocks.start()
    if ws > 1:
        dist.barrier()
    dev_ms, steps_all, res_max, launches = 0.0, [], 0.0, 0
    t0 = time.time()
    for _ in range(args.steps):
        lam, steps, res = s.solve(fac)
        ms, nl = s.stats()
        dev_ms += ms
        launches += nl
        steps_all.append(steps)
        res_max = max(res_max, float(res[:, :IEIGS].max()))
    if ws > 1:
        dist.barrier()
    wall = time.time() - t0
    clock = clocks.stop()
    t_dev = dev_ms / 1e3
    t_dev, wall = max_over_ranks([t_dev, wall])
    value = NK * ws * args.steps / t_dev

    # the last timed solve's eigenvectors, rechecked in FP64
    vec = s.eigenvectors()
    res_fp64 = fp64_residual_check(mx, n, kap, fac, lam, vec)
    del vec

    # roofline kernels: one more solve with the finest level's node GS
    # sweeps, AFW sweeps and Gram launches bracketed by CUDA events on the
    # solver's stream (the timed solves replay CUDA graphs, whose inner
    # launches carry no events)
    s.profile(True)
    s.solve(fac)
    kt = {name: s.kernel_time(q) for name, q in (("node_gs", s.KT_NODE_GS), ("afw", s.KT_AFW),
                                                 ("gram", s.KT_GRAM))}
    s.profile(False)

    # e2e: through the public API from host buffers -- solver creation
    # uploads kappa (h2d), the solve takes the k-points from host memory and
    # returns eigenvalues, step counts and residuals to host memory (d2h)
    e2e_steps = max(1, min(args.steps, 2))
    t0 = time.time()
    for _ in range(e2e_steps):
        s2 = make(1, NK)
        lam2, steps2, res2 = s2.solve(fac)
        del s2
    e2e_t = time.time() - t0
    h2d = kap.nbytes + fac.nbytes
    d2h = lam2.nbytes + steps2.nbytes + res2.nbytes
    del s

    # the plain FP64 GPU solver on the same 32 k-points in one batch of 32:
    # one untimed solve, then timed solves
    s64 = make(0, NK)
    s64.solve(fac)
    n64 = max(1, min(args.steps, 2))
    ms64 = 0.0
    for _ in range(n64):
        lam64, steps64, res64 = s64.solve(fac)
        ms64 += s64.stats()[0]
    del s64
    fp64_value = NK * n64 / (ms64 / 1e3)
    agree = float((np.abs(lam64[:, :IEIGS] - lam[:, :IEIGS]) / np.abs(lam64[:, :IEIGS])).max())

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    src = "measured" if "hbm_gbs" in peaks else "fallback (6.8 TB/s, no measured peaks)"

    def roof(name, kernel, per, traffic):
        ms, cnt, byt = kt[name]
        if not cnt:
            return None
        achieved = byt / (ms / 1e3) / 1e9
        return {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": traffic, "algorithmic_bytes": byt / cnt, "avg_ms": ms / cnt, "count": cnt,
                "per": per, "kernel": kernel, "peak_source": src}

    out = {
        "metric": METRIC, "value": value, "unit": "k-points/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64+dd",
        "data": "synthetic (disc eps=12 r=0.3 on 512^2 cells; k-points on Gamma-X-M-Gamma)",
        "config": {"workload": "512^2 disc eps=12 r=0.3, 32 k-points Gamma-X-M-Gamma, 12 pairs block 16, "
                               "LOBPCG, 7 MG levels FP32, nested iteration to 1e-2, relative residual 1e-8",
                   "k_points_per_gpu": NK, "grid": n, "pairs": IEIGS, "block": BLOCK, "levels": LEVELS + 1,
                   "l2": "working set (> 10 GB per step) far above the 129 MB L2", "device": dev,
                   "launch_shapes": dict(mx.get_tuning(), autotuned=bool(args.autotune))},
        "e2e": {"value": NK * ws * e2e_steps / e2e_t, "unit": "k-points/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "clocks": clock,
        "roofline": roof("node_gs", "k_node_gs_warp + k_node_gs_rowpar (node Gauss-Seidel of the gradient "
                                    "lifting, finest level)", "one node GS sweep (4 launches)",
                         TRAFFIC_32K["node_gs"]),
        "roofline_more": [roof("gram", "k_block_gram_split + k_gram_reduce (Gram matrices of [E X P])",
                               "one Gram of the Ritz step", TRAFFIC_32K["gram"]),
                          roof("afw", "k_edge_gs_rowpair (AFW sweep in four colours, finest level)",
                               "one AFW sweep (2 row-pair launches)", TRAFFIC_32K["afw"])],
        "fp64_gpu": {"value": fp64_value, "unit": "k-points/s", "k_points": NK, "wave": NK, "steps": n64,
                     "warmup": 1, "speedup_mixed_vs_fp64": value / fp64_value,
                     "max_rel_eig_diff_vs_mixed": agree},
        "steps_per_k": float(np.mean([st.mean() for st in steps_all])),
        "max_rel_residual": res_max,
        "max_rel_residual_fp64": res_fp64,
        "wall_s": wall,
    }
    if rank == 0 and ws == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(kap, fac, os.cpu_count() or 1, lam)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def run_reference(args):
    """The reference arm: the reference's CPU path as restated in
    oracle/maxwell_oracle.c (the reference's own sources are not on the GPU
    machine), on every host thread, following the reference driver's flow
    along the path: k-points one after the other, the first from a cold
    start (coarse eigenproblem, nested iteration), every later one
    warm-started by second-order Rayleigh-Ritz extrapolation.  Each step is
    one k-point solved to the relative residual 1e-8: the first --warmup
    k-points are untimed, the next --steps are timed one by one.  (The point
    after Gamma starts cold: the Gamma block lacks the two lowest bands of
    every k != 0.)"""
    ws, rank = dist_env()
    if rank != 0:
        return
    n = N0 << LEVELS
    kap = disc_kappa(n)
    total = args.warmup + args.steps
    fac = factors_of(gamma_x_m_gamma(max(NK, total)))[:total]
    threads = os.cpu_count() or 1
    lam, steps, res, secs = cpu_path_solve(threads, kap, fac)
    timed = secs[args.warmup:]
    v = args.steps / float(timed.sum())
    out = {"metric": METRIC, "value": v, "unit": "k-points/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * float(timed.mean()), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic (same workload)",
           "impl": "reference",
           "config": {"workload": "512^2 disc eps=12 r=0.3, k-points Gamma-X-M-Gamma, 12 pairs block 16, "
                                  "LOBPCG, 7 MG levels, relative residual 1e-8"},
           "cpu_baseline": {"value": v, "unit": "k-points/s", "cores": threads, "kind": "port",
                            "sample": (f"{args.steps} consecutive k-points of the path after {args.warmup} "
                                       f"untimed ones, each solved to relative residual 1e-8 and timed on its "
                                       f"own (block steps {', '.join(str(int(q)) for q in steps[args.warmup:])})")},
           "e2e": {"value": v, "unit": "k-points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "max_rel_residual": float(res[args.warmup:, :IEIGS].max())}
    print(json.dumps(out), flush=True)


def run_kernels(args):
    """Per-kernel roofline table of one block step's kernels at 512^2 with
    --nk k-points and block 16 (not the headline metric)."""
    import maxwell_gb300 as mx
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    rows = mx.kernel_bench(N0 << LEVELS, args.nk, BLOCK, args.reps)
    for r in rows:
        gbs = r["bytes"] / (r["ms"] / 1e3) / 1e9
        print(json.dumps({"kernel": r["name"], "n": N0 << LEVELS, "k_points": args.nk, "block": BLOCK,
                          "ms_per_call": r["ms"], "launches_per_call": r["launches"],
                          "algorithmic_bytes": r["bytes"], "achieved_gbs": gbs, "peak_gbs": hbm,
                          "frac": gbs / hbm}), flush=True)


def checkerboard_kappa(n: int, blocks: int = 16, seed: int = 0) -> np.ndarray:
    """1/eps per cell of a seeded random blocks x blocks checkerboard with eps
    drawn from {1, 4, 8.9, 12}, in the order i + j n."""
    rng = np.random.default_rng(seed)
    eps = rng.choice([1.0, 4.0, 8.9, 12.0], size=(blocks, blocks))
    return np.ascontiguousarray((1.0 / np.kron(eps, np.ones((n // blocks, n // blocks)))).reshape(-1))


def run_config5(args):
    """The large-mesh configuration: 2048^2 cells (8,388,608 edges), a seeded
    16 x 16 checkerboard of eps in {1, 4, 8.9, 12}, 8 k-points at the
    high-symmetry corners and edge midpoints (Gamma, X, Y, M, the midpoints of
    Gamma-X, Gamma-Y, Gamma-M and X-M), 24 pairs with block 32 via LOBPCG,
    9 multigrid levels 2048 .. 8 in FP32 complex, the eigenvector block in
    FP64 (precision 2), relative residual 1e-9, then one refinement sweep and
    the FP64 residual check.  Solved in two
    batches of 4 k-points (about 120 GB on the device each).  Not the
    headline metric: one JSON line."""
    import maxwell_gb300 as mx
    mx.check(mx.lib().mxg_set_device(rank_device()), "mxg_set_device")
    n0, L, ie, m, tol = 8, 8, 24, 32, 1e-9
    n = n0 << L
    kap = checkerboard_kappa(n)
    pi = np.pi
    kpts = np.array([(0, 0), (pi, 0), (0, pi), (pi, pi), (pi / 2, 0), (0, pi / 2), (pi / 2, pi / 2), (pi, pi / 2)])
    fac = factors_of(kpts)
    # FP64 eigenvector block (FP32 multigrid and search blocks): at 2048^2 the
    # float-float block's residual floor, ||A|| 2^-48 / lambda, lies above 1e-9
    s = mx.Solver(kap, n0=n0, L=L, ieigs=ie, m=m, method=1, precision=2, max_nested=MAX_NESTED,
                  nested_tol=NESTED_TOL, max_steps=120,
                  wave=4, relative=1, tol=tol, refine=1)
    ms_all, lams, steps_all, res_max, fp_max, launches = 0.0, [], [], 0.0, 0.0, 0
    for b in range(2):
        lam, st, res = s.solve(fac[4 * b:4 * b + 4])
        ms, nl = s.stats()
        ms_all += ms
        launches += nl
        fp = s.check_fp64()
        lams.append(lam[:, :ie]); steps_all += st.tolist()
        res_max = max(res_max, float(res[:, :ie].max()))
        fp_max = max(fp_max, float(fp[:, :ie].max()))
    print(json.dumps({"metric": "k-points/s, 2048^2 checkerboard, 24 pairs block 32, relative residual 1e-9",
                      "value": len(kpts) / (ms_all / 1e3), "unit": "k-points/s", "seconds": ms_all / 1e3,
                      "steps_per_k": steps_all, "max_rel_residual": res_max, "max_rel_residual_fp64": fp_max,
                      "gpu_launches": launches, "lambda_first": [float(v) for v in np.concatenate(lams)[:, 0]],
                      "config": {"workload": "2048^2, 16x16 checkerboard eps {1,4,8.9,12} seed 0, 8 k-points "
                                             "(Gamma X Y M and midpoints), 24 pairs block 32, LOBPCG, 9 levels, "
                                             "FP64 eigenvectors + FP32 multigrid, relative residual 1e-9 + "
                                             "refinement sweep + FP64 check",
                                 "batches": "2 x 4 k-points"}}), flush=True)


def run_surface(args):
    """The full-zone surface (exp_blochsurf): 256^2 cells, four discs eps = 10
    of radius 0.15 centred at (0.25|0.75, 0.25|0.75), a 32 x 32 k-grid over
    [-pi, pi]^2 solved in waves of --wave k-points (64: two rows), every wave
    after the first started as --extrapolation says (by default from the
    eigenvectors of the same slots of the wave before it), 12 pairs with
    block 16 via LOBPCG, mixed
    precision, relative residual 1e-8.  Not the headline metric: one JSON
    line of k-points/s."""
    import maxwell_gb300 as mx
    n0, L, steps, wave = 8, 5, 32, args.wave
    n = n0 << L
    h = 1.0 / n
    i = np.arange(n)
    X, Y = np.meshgrid(i * h, i * h)
    inside = np.zeros_like(X, dtype=bool)
    for cy in (0.25, 0.75):
        for cx in (0.25, 0.75):
            inside |= (X - cx) ** 2 + (Y - cy) ** 2 <= 0.15 ** 2
    kap = np.ascontiguousarray(np.where(inside, 1.0 / 10.0, 1.0).reshape(-1))
    s = mx.Solver(kap, n0=n0, L=L, ieigs=IEIGS, m=BLOCK, method=1, precision=1, max_nested=MAX_NESTED,
                  nested_tol=NESTED_TOL,
                  max_steps=60, wave=wave, relative=1, tol=TOL, extrapolation=args.extrapolation)
    for _ in range(args.warmup):
        s.solve(factors_of(gamma_x_m_gamma(wave)))
    t0 = time.time()
    lam, st, res = s.surface(steps)
    wall = time.time() - t0
    ms, nl = s.stats()
    print(json.dumps({"metric": f"k-points/s, full-zone surface 256^2, 32x32 k-grid in waves of {wave}",
                      "value": steps * steps / (ms / 1e3), "unit": "k-points/s", "wall_s": wall,
                      "steps_first_wave": float(st.reshape(-1)[:wave].mean()),
                      "steps_later_waves": float(st.reshape(-1)[wave:].mean()),
                      "max_rel_residual": float(res[..., :IEIGS].max()), "gpu_launches": nl,
                      "cold_restarts": s.restarts(),
                      "config": {"workload": f"256^2, 4 discs eps=10 r=0.15, 32x32 k-grid over the zone, "
                                             f"waves of {wave}, extrapolation '{args.extrapolation}', 12 pairs "
                                             "block 16, LOBPCG, relative residual 1e-8"}}),
          flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--kernels", action="store_true", help="per-kernel roofline table instead of the metric")
    ap.add_argument("--nk", type=int, default=NK, help="k-points of the --kernels table")
    ap.add_argument("--reps", type=int, default=5, help="timed calls per kernel of the --kernels table")
    ap.add_argument("--surface", action="store_true", help="the full-zone surface workload instead of the metric")
    ap.add_argument("--config5", action="store_true", help="the 2048^2 block-32 workload instead of the metric")
    ap.add_argument("--wave", type=int, default=64, help="k-points per wave of the --surface workload")
    ap.add_argument("--extrapolation", default="n", choices=["n", "1", "2", "c"],
                    help="start of the --surface workload's later waves: warm from the waves before "
                         "('n', or Rayleigh-Ritz over 2 or 3 waves '1', '2') or cold ('c')")
    ap.add_argument("--autotune", action="store_true",
                    help="choose the block kernels' launch shapes on the workload's sizes before warm-up")
    args = ap.parse_args()
    if args.kernels:
        run_kernels(args)
    elif args.surface:
        run_surface(args)
    elif args.config5:
        run_config5(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
