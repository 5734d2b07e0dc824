"""ctypes bindings for the two CPU oracles of the eigensolver path.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py``.  The product library never imports it.

* ``Oracle``  -> ``oracle/_build/libmaxwell_oracle.so`` (the C restatement,
  builds on any machine with gcc + OpenMP);
* ``RefLib``  -> ``oracle/_ref/libmaxwell_ref.so`` (the reference's own
  modules plus ``ref_shim.c``; only exists where the reference sources were
  available at build time).

Arrays use the reference's dense order: edge vectors hold the n*n x-edges
(i + j*n) followed by the n*n y-edges; node vectors hold n*n nodes.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libmaxwell_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libmaxwell_ref.so")

class _Cplx(C.Structure):
    """A C99 double complex passed or returned by value: on x86-64 and on
    AArch64 it travels exactly like this two-double struct."""
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


def _cz(z) -> _Cplx:
    z = complex(z)
    return _Cplx(z.real, z.imag)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def build_oracle(ref: bool = False) -> None:
    """Compile the restatement (and, if asked, the reference shim)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "restated"])
    if ref:
        subprocess.check_call(["make", "-s", "-C", HERE, "ref"])


def _cvec(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


class Oracle:
    """The C restatement (maxwell_oracle.c)."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        self.lib = C.CDLL(path)
        L = self.lib
        V, I, D = C.c_void_p, C.c_int, C.c_double
        L.om_energyprod_edge.restype = _Cplx
        L.om_massprod_edge.restype = _Cplx
        L.om_norm2.restype = D
        L.om_norm2.argtypes = [C.c_long, V]
        L.om_normmax.restype = D
        L.om_normmax.argtypes = [C.c_long, V]
        L.om_dot.restype = _Cplx
        L.om_dot.argtypes = [C.c_long, V, V]
        L.om_bloch_solve.restype = I
        L.om_bloch_solve_timed.restype = I
        L.om_rr_svqb.restype = I
        L.om_potrf.restype = I
        L.om_heev.restype = I
        L.om_hegv.restype = I
        L.om_max_threads.restype = I

    # ---- edge space ----
    def addeval_edge(self, n, kappa, xf, yf, alpha, beta, x, y):
        y = _cvec(y).copy()
        self.lib.om_addeval_edge(C.c_int(n), _p(np.ascontiguousarray(kappa, np.float64)),
                                 _cz(xf), _cz(yf), _cz(alpha), _cz(beta), _p(_cvec(x)), _p(y))
        return y

    def energyprod_edge(self, n, kappa, xf, yf, alpha, beta, x, y):
        r = self.lib.om_energyprod_edge(C.c_int(n), _p(np.ascontiguousarray(kappa, np.float64)),
                                        _cz(xf), _cz(yf), _cz(alpha), _cz(beta),
                                        _p(_cvec(x)), _p(_cvec(y)))
        return complex(r.re, r.im)

    def massprod_edge(self, n, xf, yf, x, y):
        r = self.lib.om_massprod_edge(C.c_int(n), _cz(xf), _cz(yf), _p(_cvec(x)), _p(_cvec(y)))
        return complex(r.re, r.im)

    def gs_edge(self, n, kappa, xf, yf, alpha, beta, direction, b, x):
        x = _cvec(x).copy()
        self.lib.om_gs_edge(C.c_int(n), _p(np.ascontiguousarray(kappa, np.float64)), _cz(xf), _cz(yf),
                            _cz(alpha), _cz(beta), C.c_int(direction), _p(_cvec(b)), _p(x))
        return x

    def gs_edge_simple(self, n, kappa, xf, yf, alpha, beta, direction, b, x):
        x = _cvec(x).copy()
        self.lib.om_gs_edge_simple(C.c_int(n), _p(np.ascontiguousarray(kappa, np.float64)), _cz(xf), _cz(yf),
                                   _cz(alpha), _cz(beta), C.c_int(direction), _p(_cvec(b)), _p(x))
        return x

    def gs_edge_colour(self, n, kappa, xf, yf, alpha, beta, direction, b, x):
        x = _cvec(x).copy()
        self.lib.om_gs_edge_colour(C.c_int(n), _p(np.ascontiguousarray(kappa, np.float64)), _cz(xf), _cz(yf),
                                   _cz(alpha), _cz(beta), C.c_int(direction), _p(_cvec(b)), _p(x))
        return x

    def prolong_edge(self, nc, xf, yf, alpha, c, f):
        f = _cvec(f).copy()
        self.lib.om_prolong_edge(C.c_int(nc), _cz(xf), _cz(yf), _cz(alpha), _p(_cvec(c)), _p(f))
        return f

    def restrict_edge(self, nc, xf, yf, alpha, f, c):
        c = _cvec(c).copy()
        self.lib.om_restrict_edge(C.c_int(nc), _cz(xf), _cz(yf), _cz(alpha), _p(_cvec(f)), _p(c))
        return c

    def center_edge(self, n, x):
        x = _cvec(x).copy()
        self.lib.om_center_edge(C.c_int(n), _p(x))
        return x

    def nullprod_edge(self, n, x):
        xp, yp = _Cplx(), _Cplx()
        self.lib.om_nullprod_edge(C.c_int(n), _p(_cvec(x)), C.byref(xp), C.byref(yp))
        return complex(xp.re, xp.im), complex(yp.re, yp.im)

    def nulladd_edge(self, n, xalpha, yalpha, x):
        x = _cvec(x).copy()
        self.lib.om_nulladd_edge(C.c_int(n), _cz(xalpha), _cz(yalpha), _p(x))
        return x

    def normmax(self, x):
        x = _cvec(x)
        return self.lib.om_normmax(C.c_long(x.size), _p(x))

    def center_node(self, n, v):
        v = _cvec(v).copy()
        self.lib.om_center_node(C.c_int(n), _p(v))
        return v

    def dot(self, x, y):
        x, y = _cvec(x), _cvec(y)
        r = self.lib.om_dot(C.c_long(x.size), _p(x), _p(y))
        return complex(r.re, r.im)

    def norm2(self, x):
        x = _cvec(x)
        return self.lib.om_norm2(C.c_long(x.size), _p(x))

    def dense_edge(self, n, kappa, xf, yf, alpha, beta):
        a = np.zeros((2 * n * n) ** 2, np.complex128)
        self.lib.om_dense_edge(C.c_int(n), _p(np.ascontiguousarray(kappa, np.float64)), _cz(xf), _cz(yf),
                               _cz(alpha), _cz(beta), _p(a))
        return a.reshape(2 * n * n, 2 * n * n, order="F")

    # ---- node space ----
    def addeval_node(self, n, xf, yf, alpha, x, y):
        y = _cvec(y).copy()
        self.lib.om_addeval_node(C.c_int(n), _cz(xf), _cz(yf), _cz(alpha), _p(_cvec(x)), _p(y))
        return y

    def gs_node(self, n, xf, yf, alpha, direction, b, x):
        x = _cvec(x).copy()
        self.lib.om_gs_node(C.c_int(n), _cz(xf), _cz(yf), _cz(alpha), C.c_int(direction),
                            _p(_cvec(b)), _p(x))
        return x

    def prolong_node(self, nc, xf, yf, alpha, c, f):
        f = _cvec(f).copy()
        self.lib.om_prolong_node(C.c_int(nc), _cz(xf), _cz(yf), _cz(alpha), _p(_cvec(c)), _p(f))
        return f

    def restrict_node(self, nc, xf, yf, alpha, f, c):
        c = _cvec(c).copy()
        self.lib.om_restrict_node(C.c_int(nc), _cz(xf), _cz(yf), _cz(alpha), _p(_cvec(f)), _p(c))
        return c

    def gradient(self, n, xf, yf, alpha, v, e):
        e = _cvec(e).copy()
        self.lib.om_gradient(C.c_int(n), _cz(xf), _cz(yf), _cz(alpha), _p(_cvec(v)), _p(e))
        return e

    def adjgradient(self, n, xf, yf, alpha, e, v):
        v = _cvec(v).copy()
        self.lib.om_adjgradient(C.c_int(n), _cz(xf), _cz(yf), _cz(alpha), _p(_cvec(e)), _p(v))
        return v

    def dense_node(self, n, xf, yf, fixnull):
        a = np.zeros((n * n) ** 2, np.complex128)
        self.lib.om_dense_node(C.c_int(n), _cz(xf), _cz(yf), C.c_int(int(fixnull)), _p(a))
        return a.reshape(n * n, n * n, order="F")

    # ---- grid ----
    def coarsen_kappa(self, n, kf):
        kc = np.zeros((n // 2) ** 2, np.float64)
        self.lib.om_coarsen_kappa(C.c_int(n), _p(np.ascontiguousarray(kf, np.float64)), _p(kc))
        return kc

    def disc_kappa(self, n, discs, eps_base=1.0):
        d = np.ascontiguousarray(np.asarray(discs, np.float64).reshape(-1))
        k = np.zeros(n * n, np.float64)
        self.lib.om_disc_kappa(C.c_int(n), C.c_int(len(d) // 4), _p(d), C.c_double(eps_base), _p(k))
        return k

    def pattern_kappa(self, n, rects, circles, eps_base=1.0):
        r = np.ascontiguousarray(np.asarray(rects, np.float64).reshape(-1))
        c = np.ascontiguousarray(np.asarray(circles, np.float64).reshape(-1))
        k = np.zeros(n * n, np.float64)
        self.lib.om_pattern_kappa(C.c_int(n), C.c_int(len(r) // 5), _p(r) if len(r) else None,
                                  C.c_int(len(c) // 4), _p(c) if len(c) else None, C.c_double(eps_base), _p(k))
        return k

    # ---- dense ----
    def heev(self, a):
        n = a.shape[0]
        a = np.asfortranarray(a, np.complex128).copy(order="F")
        w = np.zeros(n)
        self.lib.om_heev(C.c_int(n), _p(a), _p(w))
        return w, a

    def chol_solve(self, a, b):
        """A^-1 b by the oracle's Cholesky factorisation (om_potrf, om_potrs)."""
        n = a.shape[0]
        f = np.asfortranarray(a, np.complex128).copy(order="F")
        info = self.lib.om_potrf(C.c_int(n), _p(f))
        x = _cvec(b).copy()
        self.lib.om_potrs(C.c_int(n), _p(f), _p(x))
        return info, x

    def hegv(self, a, b):
        n = a.shape[0]
        a = np.asfortranarray(a, np.complex128).copy(order="F")
        b = np.asfortranarray(b, np.complex128).copy(order="F")
        w = np.zeros(n)
        info = self.lib.om_hegv(C.c_int(n), _p(a), _p(b), _p(w))
        return info, w, a

    # ---- multigrid ----
    def vcycle_edge(self, n0, L, kappa_fine, xf, yf, nu, coarse, cycles, b, x):
        h = self._mg(n0, L, kappa_fine, xf, yf)
        x = _cvec(x).copy()
        for _ in range(cycles):
            self.lib.om_vcycle_edge(h, C.c_int(L), C.c_int(nu), C.c_int(coarse), _p(_cvec(b)), _p(x))
        self.lib.om_mg_free(h)
        return x

    def hcycle_edge(self, n0, L, kappa_fine, xf, yf, nu, coarse, cycles, b, x):
        h = self._mg(n0, L, kappa_fine, xf, yf)
        x = _cvec(x).copy()
        for _ in range(cycles):
            self.lib.om_hcycle_edge(h, C.c_int(L), C.c_int(nu), C.c_int(coarse), _p(_cvec(b)), _p(x))
        self.lib.om_mg_free(h)
        return x

    def vcycle_node(self, n0, L, xf, yf, nu, coarse, cycles, b, x):
        n = n0 << L
        h = self._mg(n0, L, np.ones(n * n), xf, yf)
        x = _cvec(x).copy()
        for _ in range(cycles):
            self.lib.om_vcycle_node(h, C.c_int(L), C.c_int(nu), C.c_int(coarse), _p(_cvec(b)), _p(x))
        self.lib.om_mg_free(h)
        return x

    def _mg(self, n0, L, kappa_fine, xf, yf):
        self.lib.om_mg_new.restype = C.c_void_p
        h = C.c_void_p(self.lib.om_mg_new(C.c_int(n0), C.c_int(L),
                                          _p(np.ascontiguousarray(kappa_fine, np.float64))))
        self.lib.om_mg_set_bloch(h, _cz(xf), _cz(yf))
        return h

    def set_threads(self, t: int) -> None:
        self.lib.om_set_threads(C.c_int(t))

    def max_threads(self) -> int:
        return self.lib.om_max_threads()

    # ---- solver ----
    def bloch_solve(self, kappa_fine, factors, *, n0, L, ieigs, m, method=0, max_nested=20,
                    max_steps=40, prec_steps=2, gradient_steps=5, smoother_steps=2, lift_e=1,
                    center=1, extrapolation="2", wave=1, relative=1, tol=1e-8, nested_tol=0.0,
                    want_vectors=False, want_times=False):
        class Opts(C.Structure):
            _fields_ = [(f, C.c_int) for f in (
                "n0", "L", "ieigs", "m", "method", "max_nested", "max_steps", "prec_steps",
                "gradient_steps", "smoother_steps", "lift_e", "center", "extrapolation", "wave",
                "relative")] + [("tol", C.c_double), ("nested_tol", C.c_double)]
        o = Opts(n0, L, ieigs, m, method, max_nested, max_steps, prec_steps, gradient_steps,
                 smoother_steps, lift_e, center, ord(extrapolation), wave, relative, tol, nested_tol)
        factors = np.asarray(factors, np.complex128)
        nk = factors.shape[0]
        xfs = np.ascontiguousarray(factors[:, 0])
        yfs = np.ascontiguousarray(factors[:, 1])
        lam = np.zeros((nk, m))
        steps = np.zeros(nk, np.int32)
        res = np.zeros((nk, m))
        n = n0 << L
        ev = np.zeros((nk, m, 2 * n * n), np.complex128) if want_vectors else None
        secs = np.zeros(nk)
        st = self.lib.om_bloch_solve_timed(C.byref(o), _p(np.ascontiguousarray(kappa_fine, np.float64)),
                                           C.c_int(nk), _p(xfs), _p(yfs), _p(lam), _p(steps), _p(res),
                                           _p(ev) if ev is not None else None, _p(secs))
        if want_times:
            return st, lam, steps, res, ev, secs
        return st, lam, steps, res, ev

    def continuity(self, n, factors, ieigs, vertex, continuity, chern_vectors, vecs, lam):
        """om_continuity on copies: returns adjusted vectors, eigenvalues,
        Chern partial sums (nk, chern_vectors) and swap counts (nk)."""
        factors = np.asarray(factors, np.complex128)
        nk, m = vecs.shape[0], vecs.shape[1]
        v = np.ascontiguousarray(vecs, np.complex128).copy()
        lam = np.ascontiguousarray(lam, np.float64).copy()
        ch = np.zeros((nk, max(chern_vectors, 1)), np.complex128)
        sg = np.zeros(nk, np.int32)
        self.lib.om_continuity(C.c_int(n), C.c_int(nk), _p(np.ascontiguousarray(factors[:, 0])),
                               _p(np.ascontiguousarray(factors[:, 1])), C.c_int(m), C.c_int(ieigs),
                               _p(np.ascontiguousarray(vertex, np.int32)), C.c_int(ord(continuity)),
                               C.c_int(chern_vectors), _p(v), _p(lam), _p(ch), _p(sg))
        return v, lam, ch[:, :chern_vectors], sg

    def eps_sensitivity(self, n, kappa, xf, yf, vecs, weights):
        vecs = np.ascontiguousarray(vecs, np.complex128)
        w = np.ascontiguousarray(weights, np.float64)
        g = np.zeros(n * n)
        self.lib.om_eps_sensitivity(C.c_int(n), _p(np.ascontiguousarray(kappa, np.float64)),
                                    _cz(xf), _cz(yf), C.c_int(len(w)), _p(vecs), _p(w), _p(g))
        return g


class RefLib:
    """The reference's unmodified modules behind ref_shim.c."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.lib.ref_bloch_solve.restype = C.c_int

    def addeval_edge(self, n, kappa, xf, yf, alpha, beta, x, y):
        y = _cvec(y).copy()
        self.lib.ref_addeval_edge2d(C.c_int(n), _p(np.ascontiguousarray(kappa, np.float64)), _cz(xf), _cz(yf),
                                    _cz(alpha), _cz(beta), _p(_cvec(x)), _p(y))
        return y

    def products_edge(self, n, kappa, xf, yf, alpha, beta, x, y):
        out = np.zeros(3, np.complex128)
        self.lib.ref_products_edge2d(C.c_int(n), _p(np.ascontiguousarray(kappa, np.float64)), _cz(xf), _cz(yf),
                                     _cz(alpha), _cz(beta), _p(_cvec(x)), _p(_cvec(y)), _p(out))
        return out

    def gs_edge(self, n, kappa, xf, yf, alpha, beta, direction, b, x):
        x = _cvec(x).copy()
        self.lib.ref_gs_edge2d(C.c_int(n), _p(np.ascontiguousarray(kappa, np.float64)), _cz(xf), _cz(yf),
                               _cz(alpha), _cz(beta), C.c_int(direction), _p(_cvec(b)), _p(x))
        return x

    def gs_edge_simple(self, n, kappa, xf, yf, alpha, beta, direction, b, x):
        x = _cvec(x).copy()
        self.lib.ref_gs_simple_edge2d(C.c_int(n), _p(np.ascontiguousarray(kappa, np.float64)), _cz(xf), _cz(yf),
                                      _cz(alpha), _cz(beta), C.c_int(direction), _p(_cvec(b)), _p(x))
        return x

    def hcycle_edge(self, n0, L, kappa_fine, xf, yf, nu, coarse, cycles, b, x):
        x = _cvec(x).copy()
        self.lib.ref_hcycle_edge2d(C.c_int(n0), C.c_int(L), _p(np.ascontiguousarray(kappa_fine, np.float64)),
                                   _cz(xf), _cz(yf), C.c_int(nu), C.c_int(coarse), C.c_int(cycles),
                                   _p(_cvec(b)), _p(x))
        return x

    def transfer_edge(self, nc, xf, yf, alpha, restrict, a, out):
        out = _cvec(out).copy()
        self.lib.ref_transfer_edge2d(C.c_int(nc), _cz(xf), _cz(yf), _cz(alpha), C.c_int(int(restrict)),
                                     _p(_cvec(a)), _p(out))
        return out

    def addeval_node(self, n, xf, yf, alpha, x, y):
        y = _cvec(y).copy()
        self.lib.ref_addeval_node2d(C.c_int(n), _cz(xf), _cz(yf), _cz(alpha), _p(_cvec(x)), _p(y))
        return y

    def gs_node(self, n, xf, yf, alpha, direction, b, x):
        x = _cvec(x).copy()
        self.lib.ref_gs_node2d(C.c_int(n), _cz(xf), _cz(yf), _cz(alpha), C.c_int(direction),
                               _p(_cvec(b)), _p(x))
        return x

    def transfer_node(self, nc, xf, yf, alpha, restrict, a, out):
        out = _cvec(out).copy()
        self.lib.ref_transfer_node2d(C.c_int(nc), _cz(xf), _cz(yf), _cz(alpha), C.c_int(int(restrict)),
                                     _p(_cvec(a)), _p(out))
        return out

    def gradient(self, n, xf, yf, alpha, adjoint, a, out):
        out = _cvec(out).copy()
        self.lib.ref_gradient_node2d(C.c_int(n), _cz(xf), _cz(yf), _cz(alpha), C.c_int(int(adjoint)),
                                     _p(_cvec(a)), _p(out))
        return out

    def center_edge(self, n, x):
        x = _cvec(x).copy()
        self.lib.ref_center_edge2d(C.c_int(n), _p(x))
        return x

    def dense_edge(self, n, kappa, xf, yf, alpha, beta):
        a = np.zeros((2 * n * n) ** 2, np.complex128)
        self.lib.ref_densematrix_edge2d(C.c_int(n), _p(np.ascontiguousarray(kappa, np.float64)), _cz(xf),
                                        _cz(yf), _cz(alpha), _cz(beta), _p(a))
        return a.reshape(2 * n * n, 2 * n * n, order="F")

    def dense_node(self, n, xf, yf, fixnull):
        a = np.zeros((n * n) ** 2, np.complex128)
        self.lib.ref_densematrix_node2d(C.c_int(n), _cz(xf), _cz(yf), C.c_int(int(fixnull)), _p(a))
        return a.reshape(n * n, n * n, order="F")

    def coarsen_kappa(self, n0, L, kf):
        tot = sum((n0 << l) ** 2 for l in range(L + 1))
        out = np.zeros(tot)
        self.lib.ref_coarsen_kappa(C.c_int(n0), C.c_int(L), _p(np.ascontiguousarray(kf, np.float64)), _p(out))
        return out

    def vcycle_edge(self, n0, L, kappa_fine, xf, yf, nu, coarse, cycles, b, x):
        x = _cvec(x).copy()
        self.lib.ref_vcycle_edge2d(C.c_int(n0), C.c_int(L), _p(np.ascontiguousarray(kappa_fine, np.float64)),
                                   _cz(xf), _cz(yf), C.c_int(nu), C.c_int(coarse), C.c_int(cycles),
                                   _p(_cvec(b)), _p(x))
        return x

    def vcycle_node(self, n0, L, xf, yf, nu, coarse, cycles, b, x):
        x = _cvec(x).copy()
        self.lib.ref_vcycle_node2d(C.c_int(n0), C.c_int(L), _cz(xf), _cz(yf), C.c_int(nu),
                                   C.c_int(coarse), C.c_int(cycles), _p(_cvec(b)), _p(x))
        return x

    def pinvit(self, n0, L, kappa_fine, xf, yf, nu, prec, grad, lam, e):
        e = _cvec(e).copy()
        self.lib.ref_pinvit_edge2d(C.c_int(n0), C.c_int(L), _p(np.ascontiguousarray(kappa_fine, np.float64)),
                                   _cz(xf), _cz(yf), C.c_int(nu), C.c_int(prec), C.c_int(grad),
                                   C.c_double(lam), _p(e))
        return e

    def bloch_solve(self, kappa_fine, factors, *, n0, L, ieigs, throwaway, pinvit_steps,
                    bloch_steps, tol, extrapolation="2", prec_steps=2, gradient_steps=5,
                    center=1, nthreads=0):
        factors = np.asarray(factors, np.complex128)
        nk = factors.shape[0]
        m = ieigs + throwaway
        lam = np.zeros((nk, m))
        steps = np.zeros(nk, np.int32)
        dfc = np.zeros((nk, m))
        st = self.lib.ref_bloch_solve(C.c_int(n0), C.c_int(L), _p(np.ascontiguousarray(kappa_fine, np.float64)),
                                      C.c_int(nk), _p(np.ascontiguousarray(factors[:, 0])),
                                      _p(np.ascontiguousarray(factors[:, 1])), C.c_int(ieigs),
                                      C.c_int(throwaway), C.c_int(pinvit_steps), C.c_int(bloch_steps),
                                      C.c_double(tol), C.c_int(ord(extrapolation)), C.c_int(prec_steps),
                                      C.c_int(gradient_steps), C.c_int(center), C.c_int(nthreads),
                                      _p(lam), _p(steps), _p(dfc), None)
        return st, lam, steps, dfc
