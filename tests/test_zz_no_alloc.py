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


def to_device_layout(torch, x, prec):
    """A host batch [k][vector][entry] as the library's device layout
    [k][entry][vector] in the storage of prec, in a torch CUDA tensor (a
    caller's own memory)."""
    t = np.ascontiguousarray(x.transpose(0, 2, 1))
    if prec == mx.C128:
        return torch.from_numpy(t).to("cuda")
    if prec == mx.C64:
        return torch.from_numpy(t.astype(np.complex64)).to("cuda")
    hi_re = t.real.astype(np.float32)
    hi_im = t.imag.astype(np.float32)
    dd = np.stack([hi_re, (t.real - hi_re).astype(np.float32), hi_im, (t.imag - hi_im).astype(np.float32)], -1)
    return torch.from_numpy(np.ascontiguousarray(dd)).to("cuda")


def from_device_layout(t, prec):
    a = t.cpu().numpy()
    if prec == mx.CDD:
        a = (a[..., 0].astype(np.float64) + a[..., 1]) + 1j * (a[..., 2].astype(np.float64) + a[..., 3])
    return a.astype(np.complex128).transpose(0, 2, 1)


TOL = {mx.C128: 1e-13, mx.CDD: 1e-13, mx.C64: 1e-5}


@pytest.mark.parametrize("prec", [mx.C128, mx.CDD, mx.C64])
def test_noalloc_center_matches_center(prec):
    torch = pytest.importorskip("torch")
    n, m, K = 16, 3, 4
    g = mx.Grid(n, K)
    rng = np.random.default_rng(7)
    flags = torch.ones(K, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        x = rng.standard_normal((K, m, 2 * n * n)) + 1j * rng.standard_normal((K, m, 2 * n * n))
        x += (call + 1) * (0.5 - 0.25j)          # a non-zero mean in every plane
        e = mx.Edge(g, m, prec, x)
        mx.check(mx.lib().center_edge2d_gpu(e.h))
        want = e.get()
        dev = to_device_layout(torch, x, prec)
        mx.check(mx.lib().center_edge2d_gpu_noalloc(n, m, K, flags.data_ptr(), prec, dev.data_ptr(), stream))
        torch.cuda.synchronize()
        got = from_device_layout(dev, prec)
        assert rel(got, want) < TOL[prec], (call, rel(got, want))
        assert np.abs(got.reshape(K, m, 2, n * n).mean(axis=3)).max() < TOL[prec] * 10


def test_noalloc_center_at_the_limit():
    """K*m equal to MXG_CENTER_NOALLOC_MAX_KM (the whole static array)."""
    torch = pytest.importorskip("torch")
    n, m, K = 4, 32, 256
    g = mx.Grid(n, K)
    rng = np.random.default_rng(9)
    x = rng.standard_normal((K, m, 2 * n * n)) + 1j * rng.standard_normal((K, m, 2 * n * n)) + (1.0 + 2.0j)
    e = mx.Edge(g, m, mx.C128, x)
    mx.check(mx.lib().center_edge2d_gpu(e.h))
    flags = torch.ones(K, dtype=torch.int32, device="cuda")
    dev = to_device_layout(torch, x, mx.C128)
    mx.check(mx.lib().center_edge2d_gpu_noalloc(n, m, K, flags.data_ptr(), mx.C128, dev.data_ptr(),
                                                torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert rel(from_device_layout(dev, mx.C128), e.get()) < 1e-13


def test_noalloc_center_rejects_oversize():
    torch = pytest.importorskip("torch")
    flags = torch.ones(1, dtype=torch.int32, device="cuda")
    x = torch.zeros(2 * 4 * 4 * 32, dtype=torch.complex128, device="cuda")
    max_km = 8192                                   # MXG_CENTER_NOALLOC_MAX_KM
    too_many = max_km // 32 + 1
    assert mx.lib().center_edge2d_gpu_noalloc(4, 32, too_many, flags.data_ptr(), mx.C128, x.data_ptr(),
                                               None) == -1        # MXG_EINVAL, nothing launched
