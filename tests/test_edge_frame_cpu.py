"""The common-edge regular integrand of the mixed form (edge_integrand_f in
integrator2_gb300/csrc/i2_kernels_mixed.cu) restated in numpy: theta's edge terms formed in the
shared edge's frame from a point's barycentric weights, against the offset form the FP64 form
evaluates (edge_integrand in integrator2_gb300/csrc/i2_device.cuh: thetaPsi minus
singularPartAttached, evaluatorJ3DK.cu:315-350 of the reference).

- In float64 the two forms are the same function: theta and Psi agree to 1e-12 of |J| at the
  points of levels 0 and 1, over the common-edge pairs of a coarse jittered sphere (320 cells).
- In float32, over the pairs without a needle cell (a corner below 5 degrees: the mixed form
  recomputes those in FP64), the frame form keeps theta's rounding at 1.3e-7 of |J| at the 99th
  percentile and 9e-7 at most (a cell of 8 degrees); the offset form, whose vanishing terms are
  differences of offsets rounded at ulp(offset), gives 1.2e-6 and 9.6e-6.
J is the oracle's (fixed level 0); float32 here is numpy's (no fused multiply-add), a stand-in for
the kernel's rounding, not a copy of it."""
import numpy as np
import pytest

from integrator2_gb300 import meshes, pairs
from oracle import oracle as O


def _unit(v):
    return v / np.linalg.norm(v)


def _subcells(level):
    T = [np.eye(3)]
    for _ in range(level):
        nxt = []
        for a, b, c in T:
            ab, bc, ca = (a + b) / 2, (b + c) / 2, (c + a) / 2
            nxt += [np.array([a, ab, ca]), np.array([ab, b, bc]), np.array([ca, bc, c]), np.array([ab, bc, ca])]
        T = nxt
    return T


def _points(level):
    qc, qw, _ = O.QF13
    qc = np.asarray(qc, np.float64).reshape(-1, 2)
    bary = np.stack([qc[:, 0], qc[:, 1], 1.0 - qc[:, 0] - qc[:, 1]], 1)
    W = np.concatenate([bary @ U for U in _subcells(level)])           # weights of K_i's vertices
    w = np.tile(np.asarray(qw, np.float64), 4 ** level) / 4 ** level
    return W, w


def _pair_geometry(V, C, i, j):
    ci, cj = C[i], C[j]
    sj = [k for k in range(3) if cj[k] not in ci][0]
    JA, JB, JC = V[cj[sj]], V[cj[(sj + 1) % 3]], V[cj[(sj + 2) % 3]]
    kD = [k for k in range(3) if ci[k] not in cj][0]
    kB = [k for k in range(3) if ci[k] == cj[(sj + 1) % 3]][0]
    kC = 3 - kD - kB
    return JA, JB, JC, V[ci], kB, kC, kD


def offset_form(ft, V, C, i, j, W, w):
    """theta and Psi summed over the points (weights W of K_i's vertices) from the offsets to
    K_j's three vertices"""
    JA, JB, JC, Ki, _, _, _ = _pair_geometry(V, C, i, j)
    ta, tb, tc = _unit(JA - JC), _unit(JB - JA), _unit(JC - JB)
    n = np.cross(JB - JA, JC - JA)
    S2 = np.linalg.norm(n)
    f = lambda x: np.asarray(x, ft)
    ta, tb, tc, n = f(ta), f(tb), f(tc), f(n / S2)
    ilvc, S2 = ft(1.0 / np.linalg.norm(JC - JB)), ft(S2)
    Wf = f(W)
    oA, oB, oC = [Wf @ f(Ki - P) for P in (JA, JB, JC)]
    lA, lB, lC = [np.sqrt(np.sum(o * o, 1)) for o in (oA, oB, oC)]
    l1 = np.log((lA + oA @ tb) * ilvc)
    l2 = np.log((lA - oA @ ta) * ilvc)
    den = lA * lB * lC + np.sum(oA * oB, 1) * lC + np.sum(oB * oC, 1) * lA + np.sum(oC * oA, 1) * lB
    s1 = np.arctan2(np.cross(oB, tb) @ tc, (lB[:, None] * tb + oB) @ (tb - tc))
    s2 = np.arctan2(np.cross(oC, ta) @ tc, (lC[:, None] * ta - oC) @ (ta - tc))
    th = ft(2) * np.arctan2(S2 * (oA @ n), den) - ft(2) * (s1 - s2)
    psi = l1[:, None] * tb + l2[:, None] * ta
    return float(np.dot(w, th.astype(np.float64))), w @ psi.astype(np.float64)


def frame_form(ft, V, C, i, j, W, w):
    """the same sums with theta's edge terms in the shared edge's frame (constants from float64,
    rounded once, as the singular kernel stores them)"""
    JA, JB, JC, Ki, kB, kC, kD = _pair_geometry(V, C, i, j)
    ta, tb, tc = _unit(JA - JC), _unit(JB - JA), _unit(JC - JB)
    n = np.cross(JB - JA, JC - JA)
    S2 = np.linalg.norm(n)
    n = n / S2
    D = Ki[kD]
    dB = np.dot(D - JB, tc)
    Dp = (D - JB) - dB * tc
    BA = JB - JA
    f = lambda x: np.asarray(x, ft)
    L, h = ft(np.linalg.norm(JC - JB)), ft(np.linalg.norm(Dp))
    dB, dC, dn = ft(dB), ft(np.dot(JC - D, tc)), ft(np.dot(n, Dp))
    g1, g2 = ft(np.dot(Dp, np.cross(tb, tc))), ft(np.dot(Dp, np.cross(ta, tc)))
    h1, h2 = ft(np.dot(tb - tc, Dp)), ft(np.dot(ta - tc, Dp))
    cb, ca = ft(0.5 * np.dot(tb - tc, tb - tc)), ft(0.5 * np.dot(ta - tc, ta - tc))
    BAtc, BAp = ft(np.dot(BA, tc)), ft(np.dot(BA, Dp))
    ilvc, S2, taf, tbf = ft(1.0 / np.linalg.norm(JC - JB)), ft(S2), f(ta), f(tb)
    Wf = f(W)
    lBw, lCw, lD = Wf[:, kB], Wf[:, kC], Wf[:, kD]
    oA = Wf @ f(Ki - JA)
    lA = np.sqrt(np.sum(oA * oA, 1))
    l1 = np.log((lA + oA @ tbf) * ilvc)
    l2 = np.log((lA - oA @ taf) * ilvc)
    a, ap = lCw * L + lD * dB, lBw * L + lD * dC
    p2 = (lD * h) * (lD * h)
    lB, lC = np.sqrt(a * a + p2), np.sqrt(ap * ap + p2)
    inside = (a > 0) & (ap > 0)
    Q = np.where(inside, p2 * ((a * a + ap * ap + p2) / (lB * lC + a * ap)) + p2, lB * lC - a * ap + p2)
    Wt = np.where(inside, p2 * (a - ap) * (a + ap) / (lC * a + lB * ap), lC * a - lB * ap)
    den = lA * Q + (a + BAtc) * Wt + (lB + lC) * (lD * BAp + p2)
    lBa = np.where(a > 0, p2 / (lB + a), lB - a)
    lCa = np.where(ap > 0, p2 / (lC + ap), lC - ap)
    s1 = np.arctan2(lD * g1, lBa * cb + lD * h1)
    s2 = np.arctan2(lD * g2, lCa * ca - lD * h2)
    th = ft(2) * np.arctan2(S2 * (lD * dn), den) - ft(2) * (s1 - s2)
    psi = l1[:, None] * tbf + l2[:, None] * taf
    return float(np.dot(w, th.astype(np.float64))), w @ psi.astype(np.float64)


@pytest.fixture(scope="module")
def coarse():
    V, C = meshes.jittered_icosphere(2, 0.3, 11)
    pr = pairs.build_pairs(V, C).by_class(pairs.EDGE)
    e = np.linalg.norm(V[C[:, [1, 2, 0]]] - V[C], axis=2)
    la, lb, lc = e[:, 0], e[:, 1], e[:, 2]
    cos_max = np.max([(lb * lb + lc * lc - la * la) / (2 * lb * lc), (la * la + lc * lc - lb * lb) / (2 * la * lc),
                      (la * la + lb * lb - lc * lc) / (2 * la * lb)], axis=0)
    needle = cos_max > np.cos(np.radians(5.0))
    pr = pr[~(needle[pr[:, 0]] | needle[pr[:, 1]])]
    J = O.integrate(pairs.EDGE, pr, V, C, mode=O.FIXED, level=0)[1]
    S = np.array([np.linalg.norm(np.cross(V[c[1]] - V[c[0]], V[c[2]] - V[c[0]])) / 2 for c in C])
    # theta and Psi enter J as (theta n_j + Psi x n_j) / (4 pi) times K_i's area
    scale = 4 * np.pi * np.linalg.norm(J, axis=1) / S[pr[:, 0]]
    return V, C, pr, scale


@pytest.mark.parametrize("level", [0, 1])
def test_frame_form_is_the_offset_form(coarse, level):
    V, C, pr, scale = coarse
    W, w = _points(level)
    worst = 0.0
    for (i, j), s in zip(pr, scale):
        t0, p0 = offset_form(np.float64, V, C, i, j, W, w)
        t1, p1 = frame_form(np.float64, V, C, i, j, W, w)
        worst = max(worst, abs(t1 - t0) / s, np.linalg.norm(p1 - p0) / s)
    assert worst < 1e-12, worst


def test_frame_form_keeps_theta_accurate_in_float32(coarse):
    V, C, pr, scale = coarse
    W, w = _points(0)
    e_off, e_frame = [], []
    for (i, j), s in zip(pr, scale):
        t64, _ = offset_form(np.float64, V, C, i, j, W, w)
        e_off.append(abs(offset_form(np.float32, V, C, i, j, W, w)[0] - t64) / s)
        e_frame.append(abs(frame_form(np.float32, V, C, i, j, W, w)[0] - t64) / s)
    e_off, e_frame = np.array(e_off), np.array(e_frame)
    assert len(pr) > 800
    assert np.percentile(e_frame, 99) < 2e-7 and e_frame.max() < 1.5e-6, (np.percentile(e_frame, 99), e_frame.max())
    assert np.percentile(e_off, 99) > 5e-7 and e_off.max() > 5e-6, (np.percentile(e_off, 99), e_off.max())
