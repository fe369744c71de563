"""Psi of the common-vertex regular integrand in the mixed form (vertex_integrand_f and
psi_from_logs in integrator2_gb300/csrc/i2_kernels_mixed.cu) restated in numpy.  Psi is a sum of
logs along K_j's unit edges, L_bc tbc + l1 ta + l2 tb, the logs' arguments scaled by 1/sqrt(S_i).
With the unit edges and the scale rounded once to FP32 and used at every point, that rounding is
the same at every point and does not average out; summing the three logs as scalars, applying the
FP64 unit edges once per pair and taking off the integrated shift (s'/s - 1) S_i of the rounded
scale s' removes it.  On the common-vertex pairs of a coarse jittered sphere (320 cells, jitter
0.3 h; fixed level 1; leaving out the pairs the mixed form recomputes in FP64: a needle cell, or
a closed-form part 48 times J) float32 emulation gives Psi's part of J:
  per-point FP32 directions: p99 8.1e-7, 8 pairs above 1e-6 (of 2,637);
  scalar logs, FP64 directions, scale shift removed: p99 4.9e-7, 2 pairs above 1e-6.
float32 here is numpy's (no fused multiply-add), a stand-in for the kernel's rounding."""
import numpy as np
import pytest

from integrator2_gb300 import meshes, pairs
from oracle import oracle as O
from tests.test_edge_frame_cpu import _points


def _unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def _dot(a, b):
    return np.sum(a * b, axis=-1)


def _edge_log(ft, lP, qP, oP, lQ, qQ, oQ, tau, L):
    """ln((l_P + q_P) / (l_Q + q_Q)) from positive terms only (edge_log_f32's cases)"""
    s = lP + lQ
    r = np.cross(np.where((lP < lQ)[:, None], oP, oQ), tau)
    h2 = _dot(r, r)
    num = (lP + qP) * (lQ - qQ)
    c1, c2, c3 = qQ >= 0, qP <= 0, num > ft(2) * h2
    n = np.where(c1, L * (s + qP + qQ), np.where(c2, L * (s - qP - qQ), np.where(c3, num - h2, (lP + qP) * L * (s - qP - qQ))))
    d = np.where(c1, s * (lQ + qQ), np.where(c2, s * (lP - qP), np.where(c3, h2, s * h2)))
    return np.log1p(np.minimum(n / d, ft(3e38)))


@pytest.fixture(scope="module")
def coarse():
    V, C = meshes.jittered_icosphere(2, 0.3, 11)
    V, C = np.ascontiguousarray(V), np.ascontiguousarray(C, np.int32)
    pr = pairs.build_pairs(V, C).by_class(pairs.VERTEX)
    N, S, _ = O.cell_geometry(V, C)
    _, J, _, _ = O.integrate(pairs.VERTEX, pr, V, C, mode=O.FIXED, level=1)
    s4 = np.zeros((len(pr), 4))
    for k, (i, j) in enumerate(pr):
        O.lib().o_closed_vertex(int(i), int(j), O._p(V), O._p(C), O._p(N), O._p(S), O._p(s4[k]))
    nj = N[pr[:, 1]]
    ratio = np.linalg.norm(s4[:, 3:4] * nj + np.cross(s4[:, :3], nj), axis=1) / (4 * np.pi) / np.linalg.norm(J, axis=1)
    e = np.linalg.norm(V[C[:, [1, 2, 0]]] - V[C], axis=2)
    a, b, c = e[:, 0], e[:, 1], e[:, 2]
    cos_max = np.max([(b * b + c * c - a * a) / (2 * b * c), (a * a + c * c - b * b) / (2 * a * c),
                      (a * a + b * b - c * c) / (2 * a * b)], axis=0)
    keep = ~((cos_max > np.cos(np.radians(5.0)))[pr].any(axis=1) | (ratio > 48.0))
    return V, C, pr[keep], J[keep], N, S


def _psi(ft, V, C, pr, N, S, scalar_logs):
    """Psi summed over the level-1 points (times S_i), the kernel's way (scalar_logs) or with
    per-point FP32 directions"""
    ci, cj = C[pr[:, 0]], C[pr[:, 1]]
    n = len(pr)
    ar = np.arange(n)
    sj = (cj[:, :, None] == ci[:, None, :]).any(2).argmax(1)  # the shared vertex's slot in K_j
    JA, JB, JC = V[cj[ar, sj]], V[cj[ar, (sj + 1) % 3]], V[cj[ar, (sj + 2) % 3]]
    ta, tb, tbc = _unit(JA - JC), _unit(JB - JA), _unit(JC - JB)
    Si = S[pr[:, 0]]
    isq = 1.0 / np.sqrt(Si)
    f = lambda x: np.asarray(x, ft)
    cta, ctb, ctbc, cisq, cL = f(ta), f(tb), f(tbc), f(isq), f(np.linalg.norm(JC - JB, axis=1))
    T = f(V[ci] - JA[:, None, :])
    AB, AC = JB - JA, JC - JA
    ABh, ACh = f(AB), f(AC)
    ABl, ACl = f(AB - np.asarray(ABh, np.float64)), f(AC - np.asarray(ACh, np.float64))
    W, w = _points(1)
    acc = np.zeros((n, 3))
    for g in range(len(w)):
        wb = f(W[g])
        oA = wb[0] * T[:, 0] + wb[1] * T[:, 1] + wb[2] * T[:, 2]
        oB, oC = (oA - ABh) - ABl, (oA - ACh) - ACl
        lB, lC = np.sqrt(_dot(oB, oB)), np.sqrt(_dot(oC, oC))
        Lbc = _edge_log(ft, lB, _dot(oB, ctbc), oB, lC, _dot(oC, ctbc), oC, ctbc, cL)
        l1 = np.log((lC + _dot(oC, cta)) * cisq)
        l2 = np.log((lB - _dot(oB, ctb)) * cisq)
        if scalar_logs:
            acc += w[g] * np.stack([Lbc, l1, l2], 1).astype(np.float64)
        else:
            acc += w[g] * (Lbc[:, None] * ctbc + l1[:, None] * cta + l2[:, None] * ctb).astype(np.float64)
    acc *= Si[:, None]
    if not scalar_logs:
        return acc
    shift = (np.asarray(cisq, np.float64) * np.sqrt(Si) - 1.0) * Si
    return acc[:, :1] * tbc + (acc[:, 1:2] - shift[:, None]) * ta + (acc[:, 2:3] - shift[:, None]) * tb


def test_scalar_logs_with_fp64_directions(coarse):
    V, C, pr, J, N, S = coarse
    nj = N[pr[:, 1]]
    ref = _psi(np.float64, V, C, pr, N, S, False)
    scale = 4 * np.pi * np.linalg.norm(J, axis=1)

    def err(psi):
        return np.linalg.norm(np.cross(psi - ref, nj), axis=1) / scale

    e_old, e_new = err(_psi(np.float32, V, C, pr, N, S, False)), err(_psi(np.float32, V, C, pr, N, S, True))
    assert len(pr) > 2500
    assert np.percentile(e_new, 99) < 0.8 * np.percentile(e_old, 99), (np.percentile(e_new, 99), np.percentile(e_old, 99))
    assert (e_new > 1e-6).sum() < (e_old > 1e-6).sum(), ((e_new > 1e-6).sum(), (e_old > 1e-6).sum())
    # in float64 the two ways are the same function
    assert (np.linalg.norm(_psi(np.float64, V, C, pr, N, S, True) - ref, axis=1) / scale).max() < 1e-12
