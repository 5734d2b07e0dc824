"""Host side of the multi-GPU bench (one process per GPU): the k-point
partition and the max-over-ranks timing, run as two gloo ranks on CPU.  The
k-points are independent eigenproblems, so the data path has no collective;
only the timings are reduced."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        k = bench.rank_kpoints(ws, rank)
        t = bench.max_over_ranks([1.0 + rank, 10.0 - rank])
        out.put((rank, k.tolist(), t, bench.rank_device()))
    finally:
        dist.destroy_process_group()


def test_kpoint_partition_and_timing_reduction():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    sys.path.insert(0, ROOT)
    import bench
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(ws)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got.sort()
    assert [d for _, _, _, d in got] == list(range(ws))             # rank r drives GPU r
    full = bench.gamma_x_m_gamma(bench.NK * ws)
    parts = [np.array(k) for _, k, _, _ in got]
    assert all(len(p) == bench.NK for p in parts)                 # fixed work per rank
    joined = np.concatenate(parts)
    order = np.lexsort(joined.T[::-1])
    assert np.allclose(joined[order], full[np.lexsort(full.T[::-1])])   # every point exactly once
    for _, _, t, _ in got:
        assert t == [2.0, 10.0]                                     # max over ranks, element-wise
