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
