"""Permittivity adjoint (mxg_eps_sensitivity, the Hellmann-Feynman cell
reduction d lambda / d eps_c = -kappa_c^2 |curl_c e|^2 / (hx hy)) against
(1) the FP64 CPU reference gradient (the oracle's reduction on the oracle's
own eigenvectors), (2) central finite differences of the FP64 GPU solver's
eigenvalues (step 1e-6 relative, tolerance 1e-5 relative), and (3) through a
torch.autograd.Function, a band-gap objective softmin_k lambda_9 -
softmax_k lambda_8 (temperature 1e-3) against finite differences of the
objective.  Weights of eigenvalues inside a degenerate cluster are averaged
over the cluster, so every gradient here is independent of the basis the
solver picked inside a cluster."""
import numpy as np
import pytest

import maxwell_gb300 as mx

pytestmark = pytest.mark.gpu

N0, L = 8, 1
N = N0 << L
FACTORS = np.array([[np.exp(0.9j), np.exp(0.4j)], [np.exp(2.1j), np.exp(1.3j)]])
IEIGS, M = 10, 12


def random_eps(seed=3, corr=0.1):
    """1 + 11 sigmoid(g), g a periodic Gaussian random field of correlation
    length `corr` (unit-cell units), per cell."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((N, N))
    f = np.fft.fftfreq(N)[:, None] ** 2 + np.fft.fftfreq(N)[None, :] ** 2
    g = np.real(np.fft.ifft2(np.fft.fft2(w) * np.exp(-0.5 * (2 * np.pi * corr * N) ** 2 * f)))
    g = (g - g.mean()) / g.std()
    return 1.0 + 11.0 / (1.0 + np.exp(-g.reshape(-1)))


def solve(eps, want_vectors=False):
    s = mx.Solver(1.0 / eps, n0=N0, L=L, ieigs=IEIGS, m=M, method=1, precision=0, wave=len(FACTORS),
                  relative=1, tol=1e-11, max_nested=60, max_steps=100)
    lam, steps, res = s.solve(FACTORS)
    assert res[:, :IEIGS].max() <= 1e-11
    return (lam, s.eigenvectors()) if want_vectors else lam


def cluster_average(lam, w, rtol=1e-8):
    """Spread each weight evenly over the degenerate cluster it falls in."""
    w = np.array(w, dtype=np.float64)
    for k in range(lam.shape[0]):
        i = 0
        while i < lam.shape[1]:
            j = i + 1
            while j < lam.shape[1] and abs(lam[k, j] - lam[k, i]) <= rtol * abs(lam[k, i]):
                j += 1
            w[k, i:j] = w[k, i:j].mean()
            i = j
    return w


def band_weights(lam, band):
    w = np.zeros((lam.shape[0], M))
    w[:, band] = 1.0
    return cluster_average(lam[:, :M], w)


def test_adjoint_matches_cpu_reference_gradient(oracle):
    eps = random_eps()
    lam, vec = solve(eps, want_vectors=True)
    for band in (0, 3, 8):
        w = band_weights(lam, band)
        got = mx.eps_sensitivity(N, 1.0 / eps, FACTORS, vec, w)
        want = np.zeros(N * N)
        for k in range(len(FACTORS)):
            st, lam_o, _, _, vec_o = oracle.bloch_solve(1.0 / eps, FACTORS[k:k + 1], n0=N0, L=L, ieigs=IEIGS, m=M,
                                                        method=1, max_nested=60, max_steps=100, tol=1e-11,
                                                        relative=1, extrapolation="n", wave=1, want_vectors=True)
            assert st == 0
            wo = band_weights(lam_o, band)[0]
            want += oracle.eps_sensitivity(N, 1.0 / eps, *FACTORS[k], vec_o[0], wo)
        assert np.abs(got - want).max() / np.abs(want).max() < 1e-8, band


def test_adjoint_matches_finite_differences():
    eps = random_eps()
    lam, vec = solve(eps, want_vectors=True)
    band = 2
    w = band_weights(lam, band)
    adj = mx.eps_sensitivity(N, 1.0 / eps, FACTORS, vec, w)
    rng = np.random.default_rng(11)
    cells = rng.choice(N * N, 8, replace=False)
    fd = np.zeros(len(cells))
    for q, c in enumerate(cells):
        h = 1e-6 * eps[c]
        ep, em = eps.copy(), eps.copy()
        ep[c] += h
        em[c] -= h
        fd[q] = ((solve(ep)[:, :M] * w).sum() - (solve(em)[:, :M] * w).sum()) / (2 * h)
    assert np.abs(fd - adj[cells]).max() / np.abs(adj[cells]).max() < 1e-5, (fd, adj[cells])


def test_band_gap_objective_through_autograd():
    torch = pytest.importorskip("torch")
    T = 1e-3

    class Bands(torch.autograd.Function):
        """eps (cells) -> the wanted eigenvalues (k-points x IEIGS) of the FP64
        GPU solver; backward through the adjoint reduction."""

        @staticmethod
        def forward(ctx, eps_t):
            eps_np = eps_t.detach().cpu().numpy().astype(np.float64)
            lam, vec = solve(eps_np, want_vectors=True)
            ctx.save_for_backward(eps_t)
            ctx.lam, ctx.vec = lam, vec
            return torch.from_numpy(lam[:, :IEIGS].copy())

        @staticmethod
        def backward(ctx, g):
            (eps_t,) = ctx.saved_tensors
            w = np.zeros((len(FACTORS), M))
            w[:, :IEIGS] = g.detach().cpu().numpy()
            w = cluster_average(ctx.lam[:, :M], w)
            grad = mx.eps_sensitivity(N, 1.0 / eps_t.detach().cpu().numpy(), FACTORS, ctx.vec, w)
            return torch.from_numpy(grad)

    def objective(lam):
        soft_min = -T * torch.logsumexp(-lam[:, 9] / T, 0)
        soft_max = T * torch.logsumexp(lam[:, 8] / T, 0)
        return soft_min - soft_max

    eps = torch.tensor(random_eps(seed=5), dtype=torch.float64, requires_grad=True)
    obj = objective(Bands.apply(eps))
    obj.backward()
    grad = eps.grad.numpy()
    rng = np.random.default_rng(13)
    cells = rng.choice(N * N, 4, replace=False)
    base = eps.detach().numpy()
    for c in cells:
        h = 1e-6 * base[c]
        ep, em = base.copy(), base.copy()
        ep[c] += h
        em[c] -= h
        fp = objective(torch.from_numpy(solve(ep)[:, :IEIGS])).item()
        fm = objective(torch.from_numpy(solve(em)[:, :IEIGS])).item()
        fd = (fp - fm) / (2 * h)
        assert abs(fd - grad[c]) <= 1e-5 * np.abs(grad[cells]).max(), (c, fd, grad[c])


def test_config4_band_gap_gradient_full_size(oracle):
    """The differentiation configuration at its stated size: 128^2 cells,
    eps = 1 + 11 sigmoid(g) from a seeded Gaussian random field of
    correlation length 0.1, 24 k-points on Gamma-X-M-Gamma, objective
    softmin_k lambda_9 - softmax_k lambda_8 (temperature 1e-3), gradient on
    all 16,384 cells from the adjoint reduction (FP64 GPU solver).
    (1) Against the FP64 CPU reference gradient: the oracle's reduction on the
    oracle's own eigenvectors, 1e-8.  (2) Against central finite differences
    with step 1e-6 (relative to eps_c) on 64 cells drawn at random among
    those whose gradient is at least a tenth of the largest, 1e-5.  The
    objective's weights exp(-(lambda - extremum) / T) of all but the extremal
    k-points are below 1e-12 here (asserted), so the finite-difference and
    CPU solves take only the k-points above that weight; the others move the
    objective by less than 1e-12 h."""
    n0, L, ie, m, T = 8, 4, 10, 12, 1e-3
    n = n0 << L
    rng = np.random.default_rng(17)
    w = rng.standard_normal((n, n))
    f = np.fft.fftfreq(n)[:, None] ** 2 + np.fft.fftfreq(n)[None, :] ** 2
    g = np.real(np.fft.ifft2(np.fft.fft2(w) * np.exp(-0.5 * (2 * np.pi * 0.1 * n) ** 2 * f)))
    g = (g - g.mean()) / g.std()
    eps = 1.0 + 11.0 / (1.0 + np.exp(-g.reshape(-1)))
    seg = [np.pi, np.pi, np.pi * np.sqrt(2.0)]
    pts = []
    for t in np.linspace(0.0, sum(seg), 24):
        if t <= seg[0]:
            pts.append((t, 0.0))
        elif t <= seg[0] + seg[1]:
            pts.append((np.pi, t - seg[0]))
        else:
            s_ = (t - seg[0] - seg[1]) / np.sqrt(2.0)
            pts.append((np.pi - s_, np.pi - s_))
    fac = np.exp(1j * np.array(pts))

    def gpu_solve(e, f_, vectors=False):
        s = mx.Solver(1.0 / e, n0=n0, L=L, ieigs=ie, m=m, method=1, precision=0, wave=len(f_), relative=1,
                      tol=1e-11, max_nested=60, max_steps=120)
        lam, steps, res = s.solve(f_)
        assert res[:, :ie].max() <= 1e-11
        return (lam, s.eigenvectors()) if vectors else lam

    lam, vec = gpu_solve(eps, fac, True)
    wmin = np.exp(-(lam[:, 9] - lam[:, 9].min()) / T)
    wmax = np.exp((lam[:, 8] - lam[:, 8].max()) / T)
    wmin, wmax = wmin / wmin.sum(), wmax / wmax.sum()
    # d objective / d lambda: softmin weights on band 9, -softmax weights on band 8
    W = np.zeros((len(fac), m))
    W[:, 9], W[:, 8] = wmin, -wmax
    W = cluster_average(lam[:, :m], W)
    grad = mx.eps_sensitivity(n, 1.0 / eps, fac, vec, W)
    active = np.nonzero((wmin > 1e-12) | (wmax > 1e-12))[0]
    assert len(active) < len(fac)
    # (1) the CPU FP64 reference gradient on the active k-points
    want = np.zeros(n * n)
    for k in active:
        st, lam_o, _, _, vec_o = oracle.bloch_solve(1.0 / eps, fac[k:k + 1], n0=n0, L=L, ieigs=ie, m=m, method=1,
                                                    max_nested=60, max_steps=120, tol=1e-11, relative=1,
                                                    extrapolation="n", wave=1, want_vectors=True)
        assert st == 0
        wk = np.zeros((1, m))
        wk[0, 9], wk[0, 8] = wmin[k], -wmax[k]
        want += oracle.eps_sensitivity(n, 1.0 / eps, *fac[k], vec_o[0], cluster_average(lam_o[:, :m], wk)[0])
    assert np.abs(grad - want).max() / np.abs(want).max() < 1e-8

    # (2) central differences of the objective on 64 cells
    def objective(lam_active):
        full = lam.copy()
        full[active] = lam_active
        return (-T * np.log(np.exp(-(full[:, 9] - full[:, 9].min()) / T).sum()) + full[:, 9].min()
                - T * np.log(np.exp((full[:, 8] - full[:, 8].max()) / T).sum()) - full[:, 8].max())

    big = np.nonzero(np.abs(grad) >= 0.1 * np.abs(grad).max())[0]
    cells = rng.choice(big, min(64, len(big)), replace=False)
    fd = np.zeros(len(cells))
    for q, c in enumerate(cells):
        h = 1e-6 * eps[c]
        ep, em = eps.copy(), eps.copy()
        ep[c] += h
        em[c] -= h
        fd[q] = (objective(gpu_solve(ep, fac[active])) - objective(gpu_solve(em, fac[active]))) / (2 * h)
    assert np.abs(fd - grad[cells]).max() / np.abs(grad[cells]).max() < 1e-5, (fd, grad[cells])
