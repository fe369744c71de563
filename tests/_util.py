"""Shared helpers for the tests (no GPU needed to import)."""
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "integrator2_gb300.h")
GOLD = os.path.join(ROOT, "tests", "golden")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(i2_[a-z0-9_]+)\s*\(", text)))


def rel_rows(a, b):
    """per-row relative difference |a-b| / |b| (rows = pairs), guarded against tiny rows"""
    a = np.asarray(a, float).reshape(len(a), -1)
    b = np.asarray(b, float).reshape(len(b), -1)
    scale = np.maximum(np.linalg.norm(b, axis=1), 1e-12 * np.abs(b).max())
    return np.linalg.norm(a - b, axis=1) / scale


def ensure_built():
    from integrator2_gb300.build import build
    return build()


def parity_bar(kappa):
    """per-pair FP64 parity bar: 1e-12 x max(1, kappa), kappa = measured relative sensitivity of
    J to relative input perturbations.  For well-conditioned pairs this is the 1e-12 bar; for
    ill-conditioned closed forms (near-degenerate angles) the CUDA and C math libraries
    legitimately disagree in proportion to kappa."""
    return 1e-12 * np.maximum(1.0, np.asarray(kappa))


def assert_parity(J, Jref, kappa, what=""):
    r = rel_rows(J, Jref)
    bar = parity_bar(kappa)
    bad = r > bar
    assert not bad.any(), f"{what}: {bad.sum()} pairs above the bar, worst {r.max():.3e} (bar {bar[r.argmax()]:.1e})"
    return float(r.max())


def log_ratio_noise(V, C, pairs, level, J):
    """per pair: an estimate of the rounding noise of the reference's FP64 log ratios
    ln((l_P + q_P) / (l_Q + q_Q)) (evaluatorJ3DK.cu:266-313) at the 13-point rule's points of
    fixed refinement level `level`, relative to |J|.  Near the line of one of K_j's edges,
    l_Q + q_Q = l_Q (1 + r), r = unit(x - Q).tau, is a cancelling sum: its relative rounding
    error is about 2.2e-16 / (1 + r) until the reference's collinear fallback takes over at
    1 + r < 5e-13.  Summed over edges, orientations and points with the rule's |weights|, times
    the sub-cell areas and 1 / (4 pi |J|) (Psi enters J as Psi x n_j / 4 pi).  On meshes with
    nearly collinear points (the reference's cubehole.dat) it accounts for the differences
    between the reference's own host and CUDA builds."""
    from oracle import oracle as O
    qc, qw, _ = O.QF13
    qc, qw = np.asarray(qc, float).reshape(-1, 2), np.asarray(qw, float)
    bary = np.stack([qc[:, 0], qc[:, 1], 1.0 - qc[:, 0] - qc[:, 1]], 1)
    cells = [np.eye(3)]
    for _ in range(level):
        cells = [np.array(c) for t in cells for c in ((0.5 * (t[0] + t[1]), t[1], 0.5 * (t[1] + t[2])),
                                                        (0.5 * (t[1] + t[2]), t[2], 0.5 * (t[2] + t[0])),
                                                        (0.5 * (t[2] + t[0]), t[0], 0.5 * (t[0] + t[1])),
                                                        (0.5 * (t[1] + t[2]), 0.5 * (t[2] + t[0]), 0.5 * (t[0] + t[1])))]
    W = np.concatenate([bary @ U for U in cells])
    w = np.tile(qw, 4 ** level) / 4 ** level
    V, C = np.asarray(V, float), np.asarray(C)
    area = 0.5 * np.linalg.norm(np.cross(V[C[:, 1]] - V[C[:, 0]], V[C[:, 2]] - V[C[:, 0]]), axis=1)
    out = np.zeros(len(pairs))
    for t, (i, j) in enumerate(np.asarray(pairs)[:, :2]):
        X, P = W @ V[C[i]], V[C[j]]
        s = np.zeros(len(X))
        for a, b in ((0, 1), (1, 2), (2, 0)):
            tau = (P[b] - P[a]) / np.linalg.norm(P[b] - P[a])
            for to, sgn in ((P[b], 1.0), (P[a], -1.0)):
                u = X - to
                s += 2.2e-16 / np.maximum(1.0 + sgn * (u @ tau) / np.linalg.norm(u, axis=1), 5e-13)
        out[t] = (np.abs(w) @ s) * area[i] / (4.0 * np.pi * np.linalg.norm(J[t]))
    return out


def reference_checkout():
    """the reference checkout where oracle/ref_build.sh found it (it records the path in
    oracle/_ref/reference_path), or None where it was not built from one"""
    f = os.path.join(ROOT, "oracle", "_ref", "reference_path")
    if not os.path.exists(f):
        return None
    path = open(f).read().strip()
    return path if os.path.isdir(os.path.join(path, "src")) else None
