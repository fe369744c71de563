"""The potential channel and the self class have no counterpart in the reference; the oracle's
closed forms are checked here against independent adaptive quadrature (parity unpinned)."""
import numpy as np
import pytest

from oracle import oracle as O

integrate = pytest.importorskip("scipy.integrate")


def _brute_inner(x, A, B, C):
    e1, e2 = B - A, C - A
    area2 = np.linalg.norm(np.cross(e1, e2))
    f = lambda v, u: 1.0 / np.linalg.norm(x - (A + u * e1 + v * e2))
    val, _ = integrate.dblquad(f, 0, 1, 0, lambda u: 1 - u, epsabs=1e-13, epsrel=1e-12)
    return val * area2


def test_inner_potential_matches_quadrature():
    L = O.lib()
    A, B, C = np.array([0.0, 0, 0]), np.array([1.0, 0.2, 0]), np.array([0.3, 0.9, 0.1])
    for x in ([0.3, 0.3, 0.5], [0.4, 0.2, -0.3], [2.0, 1.0, 0.5], [0.5, 0.4, 0.05]):
        x = np.array(x)
        p = L.o_potential_inner(O._p(x), O._p(A), O._p(B), O._p(C))
        b = _brute_inner(x, A, B, C)
        assert abs(p - b) <= 1e-12 * abs(b)


def test_self_potential_matches_quadrature():
    L = O.lib()
    A, B, C = np.array([0.0, 0, 0]), np.array([1.0, 0.2, 0]), np.array([0.3, 0.9, 0.1])
    e1, e2 = B - A, C - A
    area2 = np.linalg.norm(np.cross(e1, e2))
    f = lambda v, u: L.o_potential_inner(O._p(A + u * e1 + v * e2), O._p(A), O._p(B), O._p(C))
    ref, _ = integrate.dblquad(f, 0, 1, 0, lambda u: 1 - u, epsabs=1e-12, epsrel=1e-11)
    ref *= area2 / (4 * np.pi)
    got = L.o_self_potential(O._p(A), O._p(B), O._p(C), 64)
    assert abs(got - ref) <= 1e-11 * ref


def test_self_potential_closed_form():
    """the closed form (4 S^2 / 3) sum_s ln(p / (p - 2 s)) / s (the library's default self rule)
    against the edge rule at 96 points per piece and against the brute-force double integral;
    exact under power-of-two rescaling (no absolute threshold); a nearly flat cell (the longest
    side within 1e-9 of the sum of the other two) stays finite and positive"""
    from integrator2_gb300 import meshes as M
    L = O.lib()
    A, B, C = np.array([0.0, 0, 0]), np.array([1.0, 0.2, 0]), np.array([0.3, 0.9, 0.1])
    e1, e2 = B - A, C - A
    area2 = np.linalg.norm(np.cross(e1, e2))
    f = lambda v, u: L.o_potential_inner(O._p(A + u * e1 + v * e2), O._p(A), O._p(B), O._p(C))
    ref, _ = integrate.dblquad(f, 0, 1, 0, lambda u: 1 - u, epsabs=1e-12, epsrel=1e-11)
    ref *= area2 / (4 * np.pi)
    assert abs(L.o_self_potential_closed(O._p(A), O._p(B), O._p(C)) - ref) <= 1e-11 * ref
    V, Cc = M.jittered_icosphere(3, 0.15, 3)
    T = np.ascontiguousarray(V[Cc], np.float64)
    closed = np.array([L.o_self_potential_closed(O._p(t[0]), O._p(t[1]), O._p(t[2])) for t in T])
    rule = np.array([L.o_self_potential(O._p(t[0]), O._p(t[1]), O._p(t[2]), 96) for t in T])
    assert np.max(np.abs(closed - rule) / rule) < 1e-12
    s = 2.0 ** -11
    Ts = np.ascontiguousarray(T * s)
    scaled = np.array([L.o_self_potential_closed(O._p(t[0]), O._p(t[1]), O._p(t[2])) for t in Ts])
    assert np.array_equal(scaled, closed * s ** 3)
    # flat cell: the direct formula in extended precision (p - 2 s formed without Heron) as reference
    flat = [np.array([0.0, 0, 0]), np.array([1.0, 0, 0]), np.array([0.5, 1e-5, 0])]
    pf = L.o_self_potential_closed(*(O._p(x) for x in flat))
    X = [x.astype(np.longdouble) for x in flat]
    a, b, c = (np.sqrt(np.sum((X[i] - X[j]) ** 2)) for i, j in ((2, 1), (0, 2), (1, 0)))
    S = np.longdouble(0.5) * np.longdouble(1e-5)
    p_ = a + b + c
    ext = (4 * S * S / 3) * (np.log(p_ / (b + c - a)) / a + np.log(p_ / (c + a - b)) / b + np.log(p_ / (a + b - c)) / c) / (4 * np.pi)
    assert np.isfinite(pf) and pf > 0 and abs(pf - float(ext)) <= 1e-9 * float(ext)


def test_potential_is_symmetric_on_a_sphere():
    """P_ij = P_ji exactly for the true integral; the discrete values agree to the quadrature error."""
    from integrator2_gb300 import meshes as M, pairs as P
    V, C = M.icosphere(2)
    pl = P.build_pairs(V, C)
    far = pl.far[:400]
    _, _, Pij, _ = O.integrate(O.FAR, far, V, C, mode=O.FIXED, level=2)
    _, _, Pji, _ = O.integrate(O.FAR, far[:, ::-1], V, C, mode=O.FIXED, level=2)
    assert np.max(np.abs(Pij - Pji) / Pij) < 1e-5
