"""center_edge2d_gpu_noalloc, the centring entry point for callers that must
not allocate device memory, against center_edge2d_gpu (which allocates its
scratch per call) on the same batches through the C ABI.  Two calls in a
row: the second one finds the first one's sums in the shared static scratch
and must clear them.  Tolerance: the 1e-13 relative of the centring test.
The device buffers come from torch, standing in for a caller's own memory."""
import numpy as np
import pytest

import maxwell_gb300 as mx

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_noalloc_center_matches_center():
    torch = pytest.importorskip("torch")
    n, m, K = 16, 3, 4
    g = mx.Grid(n, K)
    rng = np.random.default_rng(7)
    flags = torch.ones(K, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        x = rng.standard_normal((K, m, 2 * n * n)) + 1j * rng.standard_normal((K, m, 2 * n * n))
        x += (call + 1) * (0.5 - 0.25j)          # a non-zero mean in every plane
        e = mx.Edge(g, m, mx.C128, x)
        mx.check(mx.lib().center_edge2d_gpu(e.h))
        want = e.get()
        # device layout [k][entry][vector]
        dev = torch.from_numpy(np.ascontiguousarray(x.transpose(0, 2, 1))).to("cuda")
        mx.check(mx.lib().center_edge2d_gpu_noalloc(n, m, K, flags.data_ptr(), mx.C128, dev.data_ptr(), stream))
        torch.cuda.synchronize()
        got = dev.cpu().numpy().transpose(0, 2, 1)
        assert rel(got, want) < 1e-13, (call, rel(got, want))
        assert np.abs(got.reshape(K, m, 2, n * n).mean(axis=3)).max() < 1e-13


def test_noalloc_center_rejects_oversize():
    torch = pytest.importorskip("torch")
    flags = torch.ones(1, dtype=torch.int32, device="cuda")
    x = torch.zeros(2 * 4 * 4 * 32, dtype=torch.complex128, device="cuda")
    max_km = 8192                                   # MXG_CENTER_NOALLOC_MAX_KM
    too_many = max_km // 32 + 1
    assert mx.lib().center_edge2d_gpu_noalloc(4, 32, too_many, flags.data_ptr(), mx.C128, x.data_ptr(),
                                               None) == -1        # MXG_EINVAL, nothing launched
