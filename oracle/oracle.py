"""ctypes front-end of the C oracle (oracle/i2_oracle.c).  TEST INFRASTRUCTURE ONLY.

Builds liboracle.so on first use with `make -C oracle`.  Also exposes the reference-derived
host library oracle/_ref/libi2ref.so when it has been built (only possible where the reference
sources are present; see oracle/ref_build.sh).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
VERTEX, EDGE, FAR, SELF = 0, 1, 2, 3
FIXED, ADAPTIVE_COMPAT, ADAPTIVE_RELATIVE = 0, 1, 2

# Cowper's 13-point, degree-7 rule for triangles (published 15-digit table): orbits
# (centroid), 3 x (a, a, 1-2a), 6 x (a, b, 1-a-b), expanded in the published point order.
_QF13_COORDS = np.array([
    [0.333333333333333, 0.333333333333333],
    [0.479308067841923, 0.260345966079038], [0.260345966079038, 0.479308067841923],
    [0.260345966079038, 0.260345966079038],
    [0.869739794195598, 0.065130102902216], [0.065130102902216, 0.869739794195598],
    [0.065130102902216, 0.065130102902216],
    [0.638444188569809, 0.312865496004875], [0.312865496004875, 0.638444188569809],
    [0.638444188569809, 0.048690315425316], [0.048690315425316, 0.638444188569809],
    [0.312865496004875, 0.048690315425316], [0.048690315425316, 0.312865496004875]])
_QF13_W = np.array([-0.149570044467670] + [0.175615257433204] * 3 + [0.053347235608839] * 3 +
                   [0.077113760890257] * 6)
QF13 = (_QF13_COORDS, _QF13_W, 7)
# the library's default potential rule, for CPU runs doing the library's work
PRODUCT_RULE = dict(nu=10, nv=8, grade=3, adaptive=1e-8, depth=12, tiered=2e-7)

_lock = threading.Lock()
_lib = None
_ref = None


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            so = os.path.join(HERE, "liboracle.so")
            src = os.path.join(HERE, "i2_oracle.c")
            if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
                subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
            L = ctypes.CDLL(so)
            vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
            L.o_integrate_class.argtypes = [i, i, vp, vp, i, vp, i, vp, i, vp, vp, i, i, i, d, i, vp, vp, vp, vp, i]
            L.o_integrate_class.restype = i
            L.o_self_potential.argtypes = [vp, vp, vp, i]
            L.o_self_potential.restype = d
            L.o_self_potential_closed.argtypes = [vp, vp, vp]
            L.o_self_potential_closed.restype = d
            L.o_potential_inner.argtypes = [vp, vp, vp, vp]
            L.o_potential_inner.restype = d
            L.o_theta_psi.argtypes = [vp, vp, vp, vp, vp]
            L.o_task_integrand.argtypes = [i, i, i, vp, vp, i, vp, vp]
            L.o_closed_edge.argtypes = [i, i, vp, vp, vp, vp, vp]
            L.o_closed_vertex.argtypes = [i, i, vp, vp, vp, vp, vp]
            L.o_cell_geometry.argtypes = [i, vp, vp, vp, vp, vp]
            L.o_max_threads.restype = i
            L.o_set_potential_rule.argtypes = [i, i, i]
            L.o_set_potential_adaptive.argtypes = [ctypes.c_double]
            L.o_set_potential_adaptive_depth.argtypes = [i]
            L.o_set_potential_adaptive_all.argtypes = [i]
            L.o_set_potential_tiered.argtypes = [ctypes.c_double]
            L.o_pair_is_hard.argtypes = [i, i, vp, vp]
            L.o_pair_is_hard.restype = i
            L.o_adapt_stats.argtypes = [vp, i]
            L.o_set_self_rule.argtypes = [i]
            _lib = L
    return _lib


def ref_lib():
    """oracle/_ref/libi2ref.so (the reference's own routines, host build) or None."""
    global _ref
    with _lock:
        if _ref is None:
            so = os.path.join(HERE, "_ref", "libi2ref.so")
            if not os.path.exists(so):
                return None
            R = ctypes.CDLL(so)
            vp, i = ctypes.c_void_p, ctypes.c_int
            R.refd_set_qf.argtypes = [vp, vp, i, i]
            R.refd_run_class.argtypes = [i, i, vp, vp, i, vp, i, vp, i, vp, vp, vp]
            R.refd_run_class.restype = i
            R.refd_theta_psi.argtypes = [vp, vp, vp, vp, vp]
            R.refd_singular_parts.argtypes = [i, vp, i, i, i, vp, i, vp, vp]
            R.refd_closed_forms.argtypes = [i, i, i, i, vp, i, vp, vp]
            R.refd_geometry.argtypes = [i, vp, i, vp, vp, vp]
            _ref = R
    return _ref


def adapt_stats(reset=True):
    """cells visited by the adaptive potential rule per depth since the last reset"""
    out = np.zeros(32, np.int64)
    lib().o_adapt_stats(_p(out), int(reset))
    return out


def cell_geometry(V, C):
    V = np.ascontiguousarray(V, np.float64); C = np.ascontiguousarray(C, np.int32)
    n = np.empty((len(C), 3)); s = np.empty(len(C)); c = np.empty((len(C), 3))
    lib().o_cell_geometry(len(C), _p(V), _p(C), _p(n), _p(s), _p(c))
    return n, s, c


def integrate(cls, pairs, V, C, qf=QF13, mode=FIXED, level=0, tol=1e-6, self_sign=0, nthreads=0):
    """Returns (raw4 [n,4], J [n,3], P [n], levels [n])."""
    V = np.ascontiguousarray(V, np.float64)
    C = np.ascontiguousarray(C, np.int32)
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    ti = np.ascontiguousarray(pairs[:, 0]); tj = np.ascontiguousarray(pairs[:, 1])
    n = len(pairs)
    coords = np.ascontiguousarray(qf[0], np.float64); w = np.ascontiguousarray(qf[1], np.float64)
    raw = np.zeros((n, 4)); J = np.zeros((n, 3)); P = np.zeros(n); lev = np.zeros(n, np.int32)
    rc = lib().o_integrate_class(cls, n, _p(ti), _p(tj), len(V), _p(V), len(C), _p(C), len(w), _p(coords), _p(w),
                                 int(qf[2]), mode, level, tol, self_sign, _p(raw), _p(J), _p(P), _p(lev), nthreads)
    if rc != 0:
        raise ValueError(f"oracle rejected the arguments (code {rc})")
    return raw, J, P, lev


def ref_integrate(cls, pairs, V, C, level=0, qf=QF13):
    """The reference's own pipeline (host build): level >= 0 fixed (0 or 1), -1 adaptive.
    Returns (raw4, J, iters) or None when oracle/_ref is not built."""
    R = ref_lib()
    if R is None:
        return None
    coords = np.ascontiguousarray(qf[0], np.float64); w = np.ascontiguousarray(qf[1], np.float64)
    R.refd_set_qf(_p(coords), _p(w), len(w), int(qf[2]))
    V = np.ascontiguousarray(V, np.float64); C = np.ascontiguousarray(C, np.int32)
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    ti = np.ascontiguousarray(pairs[:, 0]); tj = np.ascontiguousarray(pairs[:, 1])
    n = len(pairs)
    raw = np.zeros((n, 4)); J = np.zeros((n, 3)); it = np.zeros(n, np.int32)
    rc = R.refd_run_class(cls, n, _p(ti), _p(tj), len(V), _p(V), len(C), _p(C), level, _p(raw), _p(J), _p(it))
    if rc != 0:
        raise ValueError("reference driver rejected the arguments")
    return raw, J, it


class potential_rule:
    """context manager: the oracle's adjacent-pair potential rule (Duffy nu x nv, grading) and
    adaptive hard-pair tolerance (0 = off) and the self-pair rule size; restores the high-order
    defaults on exit"""

    def __init__(self, nu=40, nv=32, grade=3, adaptive=1e-10, depth=18, every_pair=False, tiered=0.0, self_n=96):
        self.args = (nu, nv, grade, adaptive, depth, every_pair, tiered, self_n)

    def __enter__(self):
        L = lib()
        nu, nv, g, a, d, e, t, sn = self.args
        L.o_set_self_rule(sn)
        L.o_set_potential_rule(nu, nv, g)
        L.o_set_potential_adaptive(a)
        L.o_set_potential_adaptive_depth(d)
        L.o_set_potential_adaptive_all(1 if e else 0)
        L.o_set_potential_tiered(t)
        return self

    def __exit__(self, *exc):
        L = lib()
        L.o_set_potential_rule(40, 32, 3)
        L.o_set_potential_adaptive(1e-10)
        L.o_set_potential_adaptive_depth(18)
        L.o_set_potential_adaptive_all(0)
        L.o_set_potential_tiered(0.0)
        L.o_set_self_rule(96)


def hard_pairs(pairs, V, C):
    V = np.ascontiguousarray(V, np.float64); C = np.ascontiguousarray(C, np.int32)
    L = lib()
    return np.array([L.o_pair_is_hard(int(i), int(j), _p(V), _p(C)) for i, j in pairs], bool)


def conditioning(cls, pairs, V, C, level=0, rel=1e-13, seed=0):
    """per-pair sensitivity of J to relative input perturbations of size rel: the relative
    change of J divided by rel (an estimate of the condition number)"""
    V = np.ascontiguousarray(V, np.float64)
    _, J0, _, _ = integrate(cls, pairs, V, C, mode=FIXED, level=level)
    rng = np.random.default_rng(seed)
    worst = np.zeros(len(pairs))
    for _ in range(3):
        Vp = V * (1.0 + rel * rng.standard_normal(V.shape))
        _, J1, _, _ = integrate(cls, pairs, Vp, C, mode=FIXED, level=level)
        scale = np.maximum(np.linalg.norm(J0, axis=1), 1e-300)
        worst = np.maximum(worst, np.linalg.norm(J1 - J0, axis=1) / scale / rel)
    return worst
