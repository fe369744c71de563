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


def reference_checkout():
    """the reference checkout where oracle/ref_build.sh found it (it records the path in
    oracle/_ref/reference_path), or None where it was not built from one"""
    f = os.path.join(ROOT, "oracle", "_ref", "reference_path")
    if not os.path.exists(f):
        return None
    path = open(f).read().strip()
    return path if os.path.isdir(os.path.join(path, "src")) else None
