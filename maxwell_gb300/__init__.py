"""Python access to libmaxwell_gb300 (the C ABI in include/maxwell_gb300.h).

The library is the product; this module only binds it with ctypes for the
tests, the benchmark and Python callers.  It never computes anything itself
and has no fallback: if the shared library is missing, importing ``lib()``
raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmaxwell_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "maxwell_gb300.h")

C64, C128, CDD = 0, 1, 2

_lib = None


class Field(C.Structure):
    """double complex by value (same registers as a two-double struct on
    x86-64 and AArch64)."""
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


def fz(z) -> Field:
    z = complex(z)
    return Field(z.real, z.imag)


class SolveOpts(C.Structure):
    _fields_ = [(n, C.c_int) for n in (
        "n0", "L", "ieigs", "m", "method", "precision", "max_nested", "max_steps", "prec_steps",
        "gradient_steps", "smoother_steps", "lift_e", "center", "wave", "relative")] + [("tol", C.c_double),
                                                                                  ("smoother", C.c_int),
                                                                                  ("drop", C.c_double),
                                                                                  ("extrapolation", C.c_int),
                                                                                  ("refine", C.c_int),
                                                                                  ("nested_tol", C.c_double)]


class ProtocolInfo(C.Structure):
    """mxg_protocol_info (the settings in the header of the reference's
    protocol file, exp_bloch2d.c:416-443)."""
    _fields_ = [("pattern", C.c_char_p), ("n0", C.c_int), ("L", C.c_int), ("chern_vectors", C.c_int),
                ("extrapolation", C.c_int), ("stopping", C.c_int), ("continuity", C.c_int)]


def write_protocol(filename, pattern, n0, L, lam, steps=None, seconds=None, chern=None, sign=None,
                   extrapolation="2", stopping="r", continuity="s"):
    """mxg_write_protocol: the reference's protocol file of a Bloch scan."""
    lam = np.ascontiguousarray(lam, np.float64)
    nk, m = lam.shape
    cv = 0 if chern is None else np.asarray(chern).shape[1]
    info = ProtocolInfo(pattern.encode(), n0, L, cv, ord(extrapolation), ord(stopping), ord(continuity))
    arrs = [None if a is None else np.ascontiguousarray(a, t)
            for a, t in ((steps, np.int32), (seconds, np.float64), (chern, np.complex128), (sign, np.int32))]
    check(lib().mxg_write_protocol(filename.encode(), C.byref(info), nk, m, _ptr(lam),
                                   *[None if a is None else _ptr(a) for a in arrs]), "mxg_write_protocol")


class EpsPattern(C.Structure):
    """mxg_epspattern (the reference's epspattern, grid2d.h:40-62)."""
    _fields_ = [("rectangle", C.POINTER(C.c_double)), ("rectangles", C.c_int),
                ("circle", C.POINTER(C.c_double)), ("circles", C.c_int), ("eps_base", C.c_double)]


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m maxwell_gb300.build` "
                              "(or __graft_entry__.build()) first")
        L = C.CDLL(LIB_PATH)
        P, I, D, S = C.c_void_p, C.c_int, C.c_double, C.c_size_t
        protos = {
            "new_grid2d_gpu": (P, [I, I, D, D, I]),
            "del_grid2d_gpu": (None, [P]),
            "coarsen_grid2d_gpu": (P, [P]),
            "setkappa_grid2d_gpu": (I, [P, P]),
            "setbloch_grid2d_gpu": (I, [P, P, P]),
            "new_edge2d_gpu": (P, [P, I, I]),
            "del_edge2d_gpu": (None, [P]),
            "new_node2d_gpu": (P, [P, I, I]),
            "del_node2d_gpu": (None, [P]),
            "zero_edge2d_gpu": (I, [P]),
            "copy_edge2d_gpu": (I, [P, P]),
            "add_edge2d_gpu": (I, [Field, P, P]),
            "norm2_edge2d_gpu": (I, [P, P]),
            "center_edge2d_gpu": (I, [P]),
            "center_edge2d_gpu_noalloc": (I, [I, I, I, P, I, P, P]),
            "addeval_edge2d_gpu": (I, [Field, Field, P, P]),
            "addeval_shifted_edge2d_gpu": (I, [D, P, P, P]),
            "energyprod_edge2d_gpu": (I, [Field, Field, P, P, P]),
            "massprod_edge2d_gpu": (I, [P, P, P]),
            "gsforward_edge2d_gpu": (I, [Field, Field, P, P]),
            "gsbackward_edge2d_gpu": (I, [Field, Field, P, P]),
            "gssymm_edge2d_gpu": (I, [Field, Field, P, P]),
            "gscolour_edge2d_gpu": (I, [Field, Field, P, P, I]),
            "prolongation_edge2d_gpu": (I, [Field, P, P]),
            "restriction_edge2d_gpu": (I, [Field, P, P]),
            "vcycle_edge2d_gpu": (I, [I, I, P, P, P, P]),
            "densematrix_edge2d_gpu": (I, [Field, Field, P, P]),
            "denseto_edge2d_gpu": (I, [P, P]),
            "densefrom_edge2d_gpu": (I, [P, P]),
            "zero_node2d_gpu": (I, [P]),
            "addeval_node2d_gpu": (I, [Field, P, P]),
            "gsforward_node2d_gpu": (I, [Field, P, P]),
            "gsbackward_node2d_gpu": (I, [Field, P, P]),
            "gssymm_node2d_gpu": (I, [Field, P, P]),
            "prolongation_node2d_gpu": (I, [Field, P, P]),
            "restriction_node2d_gpu": (I, [Field, P, P]),
            "residual_restriction_node2d_gpu": (I, [Field, P, P, P]),
            "gradient_node2d_gpu": (I, [Field, P, P]),
            "adjgradient_node2d_gpu": (I, [Field, P, P]),
            "vcycle_node2d_gpu": (I, [I, I, P, P, P, P]),
            "densematrix_node2d_gpu": (I, [I, P, P]),
            "denseto_node2d_gpu": (I, [P, P]),
            "densefrom_node2d_gpu": (I, [P, P]),
            "new_matrix_gpu": (P, [I, I]),
            "del_matrix_gpu": (None, [P]),
            "upload_matrix_gpu": (I, [P, P]),
            "download_matrix_gpu": (I, [P, P]),
            "potrf_matrix_gpu": (I, [P, P]),
            "sygv_matrix_gpu": (I, [P, P, P, P]),
            "syev_matrix_gpu": (I, [P, P, P]),
            "mxg_solver_new": (P, [P, P]),
            "mxg_solver_free": (None, [P]),
            "mxg_bloch_solve": (I, [P, I, P, P, P, P, P]),
            "mxg_solver_eigenvectors": (I, [P, P]),
            "mxg_solver_stats": (I, [P, P, P]),
            "mxg_solver_profile": (I, [P, I]),
            "mxg_solver_kernel_time": (I, [P, I, P, P, P]),
            "mxg_eps_sensitivity": (I, [I, P, I, P, P, I, P, P, P]),
            "mxg_device_ok": (I, []),
            "mxg_set_device": (I, [I]),
            "mxg_solver_restarts": (I, [P]),
            "mxg_solver_check_fp64": (I, [P, P]),
            "mxg_bloch_continuity": (I, [P, I, P, I, I, P, P, P]),
            "gsforward_simple_edge2d_gpu": (I, [Field, Field, P, P]),
            "gsbackward_simple_edge2d_gpu": (I, [Field, Field, P, P]),
            "gssymm_simple_edge2d_gpu": (I, [Field, Field, P, P]),
            "hcycle_edge2d_gpu": (I, [I, I, P, P, P, P, P, P]),
            "mxg_write_protocol": (I, [C.c_char_p, P, I, I, P, P, P, P, P]),
            "mxg_get_tuning": (I, [P]),
            "mxg_set_tuning": (I, [P]),
            "mxg_autotune": (I, [I, I, I, I, P]),
            "mxg_bloch_surface": (I, [P, I, P, P, P]),
            "mxg_kernel_bench": (I, [I, I, I, I, P, I]),
            "swap_edge2d_gpu": (I, [P, P]),
            "random_edge2d_gpu": (I, [P, C.c_ulonglong]),
            "scale_edge2d_gpu": (I, [Field, P]),
            "normmax_edge2d_gpu": (I, [P, P]),
            "dotprod_edge2d_gpu": (I, [P, P, P]),
            "nullprod_edge2d_gpu": (I, [P, P, P]),
            "nulladd_edge2d_gpu": (I, [P, P, P]),
            "gram_edge2d_gpu": (I, [P, P, P]),
            "lincomb_edge2d_gpu": (I, [P, P, P]),
            "orthonormalize_edge2d_gpu": (I, [P, P]),
            "pinvit_edge2d_gpu": (I, [I, I, I, I, P, P, P, P, P, P, P, P, P, P]),
            "copy_node2d_gpu": (I, [P, P]),
            "random_node2d_gpu": (I, [P, C.c_ulonglong]),
            "scale_node2d_gpu": (I, [Field, P]),
            "add_node2d_gpu": (I, [Field, P, P]),
            "norm2_node2d_gpu": (I, [P, P]),
            "normmax_node2d_gpu": (I, [P, P]),
            "dotprod_node2d_gpu": (I, [P, P, P]),
            "center_node2d_gpu": (I, [P]),
            "potrsv_matrix_gpu": (I, [P, P]),
            "new_epspattern_gpu": (P, [D, I, I]),
            "del_epspattern_gpu": (None, [P]),
            "setpattern_grid2d_gpu": (I, [P, P]),
            "getkappa_grid2d_gpu": (I, [P, P]),
            "getsize_grid2d_gpu": (I, [P, P, P]),
        }
        for name, (res, args) in protos.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def check(code: int, what: str = "call") -> None:
    if code != 0:
        raise RuntimeError(f"libmaxwell_gb300 {what} failed with status {code}")


class KBenchRow(C.Structure):
    _fields_ = [("name", C.c_char * 40), ("ms", C.c_double), ("bytes", C.c_double), ("launches", C.c_int)]


def kernel_bench(n: int, K: int, m: int, reps: int = 5) -> list[dict]:
    """Per-kernel timing of one block step's hot kernels (mxg_kernel_bench):
    name, mean ms per call, algorithmic bytes per call, launches per call."""
    rows = (KBenchRow * 32)()
    r = lib().mxg_kernel_bench(n, K, m, reps, rows, 32)
    if r < 0:
        raise RuntimeError(f"mxg_kernel_bench failed: {r}")
    return [{"name": rows[i].name.decode(), "ms": rows[i].ms, "bytes": rows[i].bytes,
             "launches": rows[i].launches} for i in range(r)]


class Tuning(C.Structure):
    """mxg_tuning: launch shapes of the block kernels."""
    _fields_ = [("gram_waves", C.c_int), ("combine_ctas", C.c_int), ("residual_sites", C.c_int),
                ("node_strip", C.c_int), ("node_band", C.c_int), ("restrict_strip_log2", C.c_int)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


def autotune(n: int, K: int, m: int, reps: int = 3) -> dict:
    """mxg_autotune: choose the launch shapes for n x n cells, K k-points,
    block m, and keep them for this process."""
    t = Tuning()
    r = lib().mxg_autotune(n, K, m, reps, C.byref(t))
    if r != 0:
        raise RuntimeError(f"mxg_autotune failed: {r}")
    return t.as_dict()


def get_tuning() -> dict:
    t = Tuning()
    check(lib().mxg_get_tuning(C.byref(t)), "mxg_get_tuning")
    return t.as_dict()


def set_tuning(gram_waves: int, combine_ctas: int, residual_sites: int, node_strip: int = 0,
               node_band: int = 16, restrict_strip_log2: int = 25) -> None:
    t = Tuning(gram_waves, combine_ctas, residual_sites, node_strip, node_band, restrict_strip_log2)
    check(lib().mxg_set_tuning(C.byref(t)), "mxg_set_tuning")


def header_functions() -> list[str]:
    """Names of the functions declared in include/maxwell_gb300.h."""
    import re
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", txt)
    skip = {"if", "sizeof", "return"}
    out = []
    for n in names:
        if n in skip or n.isupper():
            continue
        if n not in out:
            out.append(n)
    return out


# ----------------------------------------------------------------------
# thin object wrappers used by the tests
# ----------------------------------------------------------------------
class Grid:
    def __init__(self, n: int, K: int = 1, kappa=None, factors=None, _handle=None):
        self.n, self.K = n, K
        self.h = _handle if _handle is not None else lib().new_grid2d_gpu(n, n, 1.0 / n, 1.0 / n, K)
        if not self.h:
            raise RuntimeError("new_grid2d_gpu failed")
        if kappa is not None:
            check(lib().setkappa_grid2d_gpu(self.h, _ptr(np.ascontiguousarray(kappa, np.float64))), "setkappa")
        if factors is not None:
            self.set_bloch(factors)

    def set_bloch(self, factors):
        f = np.asarray(factors, np.complex128).reshape(self.K, 2)
        xf, yf = np.ascontiguousarray(f[:, 0]), np.ascontiguousarray(f[:, 1])
        check(lib().setbloch_grid2d_gpu(self.h, _ptr(xf), _ptr(yf)), "setbloch")

    def set_pattern(self, rects, circles, eps_base=1.0):
        """setpattern_grid2d_gpu: rectangles (eps, x0, y0, w, h), circles (eps, cx, cy, r)."""
        rects = np.asarray(rects, np.float64).reshape(-1, 5)
        circles = np.asarray(circles, np.float64).reshape(-1, 4)
        p = lib().new_epspattern_gpu(float(eps_base), len(rects), len(circles))
        if not p:
            raise RuntimeError("new_epspattern_gpu failed")
        try:
            pat = C.cast(p, C.POINTER(EpsPattern)).contents
            for q, v in enumerate(rects.reshape(-1)):
                pat.rectangle[q] = v
            for q, v in enumerate(circles.reshape(-1)):
                pat.circle[q] = v
            check(lib().setpattern_grid2d_gpu(p, self.h), "setpattern_grid2d")
        finally:
            lib().del_epspattern_gpu(p)

    def kappa(self) -> np.ndarray:
        k = np.zeros(self.n * self.n)
        check(lib().getkappa_grid2d_gpu(self.h, _ptr(k)), "getkappa_grid2d")
        return k

    def coarsen(self) -> "Grid":
        h = lib().coarsen_grid2d_gpu(self.h)
        return Grid(self.n // 2, self.K, _handle=h)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.del_grid2d_gpu(self.h)


class Edge:
    def __init__(self, g: Grid, m: int = 1, prec: int = C128, data=None):
        self.g, self.m, self.prec = g, m, prec
        self.h = lib().new_edge2d_gpu(g.h, m, prec)
        if not self.h:
            raise RuntimeError("new_edge2d_gpu failed")
        if data is not None:
            self.put(data)

    @property
    def shape(self):
        return (self.g.K, self.m, 2 * self.g.n * self.g.n)

    def put(self, data):
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(data, np.complex128), self.shape))
        check(lib().denseto_edge2d_gpu(_ptr(a), self.h), "denseto_edge2d")

    def get(self) -> np.ndarray:
        a = np.zeros(self.shape, np.complex128)
        check(lib().densefrom_edge2d_gpu(self.h, _ptr(a)), "densefrom_edge2d")
        return a

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.del_edge2d_gpu(self.h)


class Node:
    def __init__(self, g: Grid, m: int = 1, prec: int = C128, data=None):
        self.g, self.m, self.prec = g, m, prec
        self.h = lib().new_node2d_gpu(g.h, m, prec)
        if not self.h:
            raise RuntimeError("new_node2d_gpu failed")
        if data is not None:
            self.put(data)

    @property
    def shape(self):
        return (self.g.K, self.m, self.g.n * self.g.n)

    def put(self, data):
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(data, np.complex128), self.shape))
        check(lib().denseto_node2d_gpu(_ptr(a), self.h), "denseto_node2d")

    def get(self) -> np.ndarray:
        a = np.zeros(self.shape, np.complex128)
        check(lib().densefrom_node2d_gpu(self.h, _ptr(a)), "densefrom_node2d")
        return a

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.del_node2d_gpu(self.h)


class Matrix:
    def __init__(self, rows: int, K: int = 1):
        self.rows, self.K = rows, K
        self.h = lib().new_matrix_gpu(rows, K)
        if not self.h:
            raise RuntimeError("new_matrix_gpu failed")

    def get(self) -> np.ndarray:
        a = np.zeros((self.K, self.rows, self.rows), np.complex128)
        check(lib().download_matrix_gpu(self.h, _ptr(a)), "download_matrix")
        return np.transpose(a, (0, 2, 1))   # column-major per k

    def put(self, a):
        a = np.ascontiguousarray(np.transpose(np.asarray(a, np.complex128).reshape(self.K, self.rows, self.rows), (0, 2, 1)))
        check(lib().upload_matrix_gpu(self.h, _ptr(a)), "upload_matrix")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.del_matrix_gpu(self.h)


class Solver:
    """The batched per-k eigensolver (mxg_bloch_solve)."""

    def __init__(self, kappa_fine, *, n0, L, ieigs, m, method=1, precision=1, max_nested=20,
                 max_steps=60, prec_steps=2, gradient_steps=5, smoother_steps=2, lift_e=1, center=1,
                 wave=1, relative=1, tol=1e-8, smoother=1, drop=0.0, extrapolation="n", refine=0,
                 nested_tol=0.0):
        self.o = SolveOpts(n0, L, ieigs, m, method, precision, max_nested, max_steps, prec_steps,
                           gradient_steps, smoother_steps, lift_e, center, wave, relative, tol, smoother, drop,
                           ord(extrapolation), refine, nested_tol)
        self.n = n0 << L
        self.m, self.wave = m, wave
        k = np.ascontiguousarray(kappa_fine, np.float64)
        self.h = lib().mxg_solver_new(C.byref(self.o), _ptr(k))
        if not self.h:
            raise RuntimeError("mxg_solver_new failed (bad options or out of device memory)")

    def solve(self, factors):
        f = np.asarray(factors, np.complex128).reshape(-1, 2)
        nk = f.shape[0]
        xf, yf = np.ascontiguousarray(f[:, 0]), np.ascontiguousarray(f[:, 1])
        lam = np.zeros((nk, self.m))
        steps = np.zeros(nk, np.int32)
        res = np.zeros((nk, self.m))
        check(lib().mxg_bloch_solve(self.h, nk, _ptr(xf), _ptr(yf), _ptr(lam), _ptr(steps), _ptr(res)),
              "mxg_bloch_solve")
        return lam, steps, res

    def surface(self, steps: int):
        """exp_blochsurf's full-zone grid (mxg_bloch_surface): eigenvalues
        (steps, steps, m) indexed [iy, ix], block steps (steps, steps) and
        residuals (steps, steps, m)."""
        nk = steps * steps
        lam = np.zeros((nk, self.m))
        st = np.zeros(nk, np.int32)
        res = np.zeros((nk, self.m))
        check(lib().mxg_bloch_surface(self.h, steps, _ptr(lam), _ptr(st), _ptr(res)), "mxg_bloch_surface")
        return lam.reshape(steps, steps, self.m), st.reshape(steps, steps), res.reshape(steps, steps, self.m)

    def eigenvectors(self) -> np.ndarray:
        a = np.zeros((self.wave, self.m, 2 * self.n * self.n), np.complex128)
        check(lib().mxg_solver_eigenvectors(self.h, _ptr(a)), "eigenvectors")
        return a

    def stats(self):
        ms, launches = C.c_double(0), C.c_long(0)
        lib().mxg_solver_stats(self.h, C.byref(ms), C.byref(launches))
        return ms.value, launches.value

    def continuity(self, lam, vertex, continuity="s", chern_vectors=0):
        """mxg_bloch_continuity on the last solve: returns the reordered
        eigenvalues, the Chern partial sums (nk, chern_vectors) and the swap
        counts (nk)."""
        lam = np.ascontiguousarray(np.array(lam, np.float64))
        nk = lam.shape[0]
        v = np.ascontiguousarray(np.asarray(vertex, np.int32))
        ch = np.zeros((nk, max(chern_vectors, 1)), np.complex128)
        sg = np.zeros(nk, np.int32)
        check(lib().mxg_bloch_continuity(self.h, nk, _ptr(v), ord(continuity), chern_vectors, _ptr(lam), _ptr(ch),
                                          _ptr(sg)), "mxg_bloch_continuity")
        return lam, ch[:, :chern_vectors], sg

    def check_fp64(self) -> np.ndarray:
        """Relative residuals of the last wave recomputed in FP64 (wave, m)."""
        r = np.zeros(self.wave * self.m)
        check(lib().mxg_solver_check_fp64(self.h, _ptr(r)), "mxg_solver_check_fp64")
        return r.reshape(self.wave, self.m)

    def restarts(self) -> int:
        """Warm-started waves of the last solve that were solved again cold."""
        return lib().mxg_solver_restarts(self.h)

    def profile(self, enable: bool = True):
        check(lib().mxg_solver_profile(self.h, int(enable)), "profile")

    KT_NODE_GS, KT_AFW, KT_GRAM = 0, 1, 2

    def kernel_time(self, which: int = 0):
        """(summed ms, count, summed algorithmic bytes) of the finest
        level's node GS sweeps (0), AFW sweeps (1) or Gram launches (2)
        since profile(True)."""
        ms, cnt, b = C.c_double(0), C.c_long(0), C.c_double(0)
        check(lib().mxg_solver_kernel_time(self.h, which, C.byref(ms), C.byref(cnt), C.byref(b)), "kernel_time")
        return ms.value, cnt.value, b.value

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.mxg_solver_free(self.h)


def eps_sensitivity(n, kappa, factors, vecs, weights):
    f = np.asarray(factors, np.complex128).reshape(-1, 2)
    nk = f.shape[0]
    vecs = np.ascontiguousarray(vecs, np.complex128)
    m = vecs.shape[1]
    w = np.ascontiguousarray(weights, np.float64).reshape(nk * m)
    g = np.zeros(n * n)
    xf, yf = np.ascontiguousarray(f[:, 0]), np.ascontiguousarray(f[:, 1])
    check(lib().mxg_eps_sensitivity(n, _ptr(np.ascontiguousarray(kappa, np.float64)), nk, _ptr(xf), _ptr(yf),
                                    m, _ptr(vecs), _ptr(w), _ptr(g)), "mxg_eps_sensitivity")
    return g
