"""Benchmark: k-points/s of the Bloch eigensolver at 512^2, 12 eigenpairs to a
relative residual of 1e-8 (mixed precision, batched over k-points) next to
the plain FP64 GPU solver and the CPU oracle.

Workload (one "step" = one complete solve of the batch): the unit cell
meshed as 512 x 512 cells, eps = 12 inside the centred disc of radius 0.3,
eps = 1 outside; 32 Bloch k-points spaced evenly in arc length along
Gamma-X-M-Gamma; 12 wanted pairs with block 16 via LOBPCG; 7 multigrid levels
(512 .. 8) in FP32 complex; Gram, Cholesky-QR and Ritz in FP64-accurate
arithmetic; stopping rule relative residual <= 1e-8 for every wanted pair.
Every step solves the 32 k-points from scratch (coarse eigenproblem, nested
iteration, LOBPCG), so no step can reuse another's results.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank solves its own 32 k-points (rank r takes every N-th
point of a 32*N-point path): per-GPU work is fixed, no data-path collective.
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
            self.proc = subprocess.Popen(["nvidia-smi", "-i", os.environ.get("LOCAL_RANK", "0"),
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


# nested iteration: at most 5 block steps per coarse level, the reference's
# default (exp_bloch2d.c:298, pinvit_steps)
MAX_NESTED = 5
CPU_KW = dict(n0=N0, L=LEVELS, ieigs=IEIGS, m=BLOCK, method=1, max_nested=MAX_NESTED, relative=1, tol=TOL,
              extrapolation="n", wave=1)


def cpu_setup_time(O, kap, fac) -> float:
    """One k-point of the oracle up to the first block step: coarse
    eigenproblem and nested iteration (<= MAX_NESTED steps per level)."""
    t0 = time.time()
    O.bloch_solve(kap, fac[:1], max_steps=0, **CPU_KW)
    return time.time() - t0


def cpu_sample(O, kap, fac, t_setup: float, threads: int, steps_per_k: float) -> dict:
    """The oracle port (oracle/maxwell_oracle.c, OpenMP on `threads` host
    threads) on a bounded sample of the same workload: one k-point through
    the setup and 2 LOBPCG steps at 512^2.  The time per k-point is the setup
    plus `steps_per_k` block steps at the sampled step time."""
    t0 = time.time()
    O.bloch_solve(kap, fac[:1], max_steps=2, **CPU_KW)
    t_two = time.time() - t0
    t_step = max((t_two - t_setup) / 2.0, 1e-9)
    per_k = t_setup + t_step * steps_per_k
    return {"value": 1.0 / per_k, "unit": "k-points/s", "cores": threads, "kind": "port",
            "sample": (f"1 k-point at 512^2: setup (coarse eigenproblem + nested iteration, <=5 steps per "
                       f"level) {t_setup:.1f} s, 2 LOBPCG steps {2 * t_step:.1f} s; per k-point = setup + "
                       f"{steps_per_k:.1f} steps x step time")}


def cpu_baseline(kap, fac, threads: int, steps_per_k: float) -> dict:
    O = _oracle(threads)
    return cpu_sample(O, kap, fac, cpu_setup_time(O, kap, fac), threads, steps_per_k)


def run_ours(args):
    import maxwell_gb300 as mx
    ws, rank = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if not mx.lib().mxg_device_ok():
        raise RuntimeError("no CUDA device")
    n = N0 << LEVELS
    kap = disc_kappa(n)
    kpts = rank_kpoints(ws, rank)
    fac = factors_of(kpts)

    def make(precision, wave):
        return mx.Solver(kap, n0=N0, L=LEVELS, ieigs=IEIGS, m=BLOCK, method=1, precision=precision,
                         max_nested=MAX_NESTED, max_steps=60, wave=wave, relative=1, tol=TOL)

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
    wall = time.time() - t0
    clock = clocks.stop()
    t_dev = dev_ms / 1e3
    t_dev, wall = max_over_ranks([t_dev, wall])
    value = NK * ws * args.steps / t_dev

    # the roofline kernel: one more solve with its finest-level AFW sweeps
    # bracketed by CUDA events on the solver's stream (the timed solves above
    # replay CUDA graphs, whose inner launches carry no events)
    s.profile(True)
    s.solve(fac)
    kms, kcount, kbytes = s.kernel_time()
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

    # plain FP64 GPU solver on the first 8 k-points (same metric)
    n64 = 8
    s64 = make(0, n64)
    lam64, steps64, res64 = s64.solve(fac[:n64])
    ms64, _ = s64.stats()
    fp64_value = n64 / (ms64 / 1e3)
    agree = float(np.abs(lam64[:, :IEIGS] - lam[:n64, :IEIGS]).max() / np.abs(lam64[:, :IEIGS]).max())

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    # DRAM bytes of one AFW sweep at 512^2 x 32 k x 16 vectors:
    # dram__bytes_read.sum + dram__bytes_write.sum of one row-pair launch at
    # 4 k-points (648.1 MB, one ncu capture), x 8 for 32 k-points, x 2 launches
    traffic_per_sweep = 2 * 648.1e6 * (NK / 4)
    avg_s = (kms / 1e3) / max(kcount, 1)
    achieved = kbytes / avg_s / 1e9 if kcount else None
    out = {
        "metric": METRIC, "value": value, "unit": "k-points/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64+dd",
        "data": "synthetic (disc eps=12 r=0.3 on 512^2 cells; k-points on Gamma-X-M-Gamma)",
        "config": {"workload": "512^2 disc eps=12 r=0.3, 32 k-points Gamma-X-M-Gamma, 12 pairs block 16, "
                               "LOBPCG, 7 MG levels FP32, relative residual 1e-8",
                   "k_points_per_gpu": NK, "grid": n, "pairs": IEIGS, "block": BLOCK, "levels": LEVELS + 1,
                   "l2": "working set (> 10 GB per step) far above the 129 MB L2"},
        "e2e": {"value": NK * ws * e2e_steps / e2e_t, "unit": "k-points/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "clocks": clock,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None, "traffic": traffic_per_sweep,
                     "per": "one AFW sweep (2 row-pair launches)", "algorithmic_bytes": kbytes,
                     "kernel": "k_edge_gs_rowpair (AFW sweep in four colours, paired by vertex-row parity, "
                               "finest level)",
                     "peak_source": "measured" if "hbm_gbs" in peaks else "fallback (6.8 TB/s, no measured peaks)"},
        "fp64_gpu": {"value": fp64_value, "unit": "k-points/s", "k_points": n64,
                     "speedup_mixed_vs_fp64": value / fp64_value, "max_rel_eig_diff_vs_mixed": agree},
        "steps_per_k": float(np.mean([st.mean() for st in steps_all])),
        "max_rel_residual": res_max,
        "wall_s": wall,
    }
    if rank == 0 and ws == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(kap, fac, os.cpu_count() or 1, out["steps_per_k"])
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_reference(args):
    """The reference arm: the reference's CPU path as restated in
    oracle/maxwell_oracle.c (the reference's own sources are not on the GPU
    machine), on every host thread.  Warm-up: one setup-only sample (its time
    enters every step's extrapolation); each timed step: one bounded sample
    of the same workload (one k-point, setup and 2 LOBPCG steps)."""
    ws, rank = dist_env()
    if rank != 0:
        return
    n = N0 << LEVELS
    kap = disc_kappa(n)
    fac = factors_of(gamma_x_m_gamma(NK))
    threads = os.cpu_count() or 1
    # block steps per k-point that the GPU LOBPCG needs on this workload (11-13)
    steps_per_k = 12.0
    O = _oracle(threads)
    t_setup = cpu_setup_time(O, kap, fac)
    vals = [cpu_sample(O, kap, fac, t_setup, threads, steps_per_k) for _ in range(args.steps)]
    v = float(np.mean([c["value"] for c in vals]))
    out = {"metric": METRIC, "value": v, "unit": "k-points/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 / v, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "c128", "data": "synthetic (same workload)", "impl": "reference",
           "config": {"workload": "512^2 disc eps=12 r=0.3, 32 k-points Gamma-X-M-Gamma, 12 pairs block 16, "
                                  "LOBPCG, 7 MG levels, relative residual 1e-8"},
           "cpu_baseline": {"value": v, "unit": "k-points/s", "cores": threads, "kind": "port",
                            "sample": vals[-1]["sample"]},
           "e2e": {"value": v, "unit": "k-points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
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


def run_surface(args):
    """The full-zone surface (exp_blochsurf): 256^2 cells, four discs eps = 10
    of radius 0.15 centred at (0.25|0.75, 0.25|0.75), a 32 x 32 k-grid over
    [-pi, pi]^2 solved in waves of 64 (each wave starting from the previous
    one), 12 pairs with block 16 via LOBPCG, mixed precision, relative
    residual 1e-8.  Not the headline metric: one JSON line of k-points/s."""
    import maxwell_gb300 as mx
    n0, L, steps, wave = 8, 5, 32, 64
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
                  max_steps=60, wave=wave, relative=1, tol=TOL)
    for _ in range(args.warmup):
        s.solve(factors_of(gamma_x_m_gamma(wave)))
    t0 = time.time()
    lam, st, res = s.surface(steps)
    wall = time.time() - t0
    ms, nl = s.stats()
    print(json.dumps({"metric": "k-points/s, full-zone surface 256^2, 32x32 k-grid in waves of 64",
                      "value": steps * steps / (ms / 1e3), "unit": "k-points/s", "wall_s": wall,
                      "steps_first_wave": float(st.reshape(-1)[:wave].mean()),
                      "steps_later_waves": float(st.reshape(-1)[wave:].mean()),
                      "max_rel_residual": float(res[..., :IEIGS].max()), "gpu_launches": nl,
                      "config": {"workload": "256^2, 4 discs eps=10 r=0.15, 32x32 k-grid over the zone, "
                                             "waves of 64, 12 pairs block 16, LOBPCG, relative residual 1e-8"}}),
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
    args = ap.parse_args()
    if args.kernels:
        run_kernels(args)
    elif args.surface:
        run_surface(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
