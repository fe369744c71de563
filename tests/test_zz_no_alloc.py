"""The entry point that allocates nothing (i2_not_neighbors_noalloc), called through the C-ABI
with caller-owned device buffers, against the evaluator's device entry point on the same pairs
(disjoint class, relative error control, 13-point rule): per-pair relative difference within
the FP64 parity bar of 1e-12, on two calls in a row that share the static scratch array.
Collected last on purpose: it must pass both alone in a fresh process and after every other
test."""
import ctypes

import numpy as np
import pytest

from tests._util import ensure_built, rel_rows

pytestmark = pytest.mark.gpu

TOL = 1e-12
I2_ERR_INVALID_ARGUMENT = 1
MAX_CELLS, MAX_PAIRS = 8192, 16384


def _existing(api, V, C, pairs, tol, max_level):
    m = api.Mesh3D()
    m.setGeometry(V, C)
    m.prepareMesh(3.0)
    it = api.NumericalIntegrator3D(m, api.qf3D13)
    it.setErrorControl(api.RELATIVE_ERROR_CONTROL, tol, max_level)
    ev = api.EvaluatorJ3DK(m, it)
    ev.runClass(2, pairs)
    return ev.getResults(2), ev.getPotentials(2)


def _noalloc(lib, torch, dV, dC, pairs, tol, max_level):
    dpairs = torch.from_numpy(np.ascontiguousarray(pairs, np.int32)).cuda()
    n = len(pairs)
    dJ = torch.full((n, 3), float("nan"), dtype=torch.float64, device="cuda")
    dP = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    st = lib.i2_not_neighbors_noalloc(ctypes.c_void_p(dV.data_ptr()), dV.shape[0], ctypes.c_void_p(dC.data_ptr()),
                                      dC.shape[0], ctypes.c_void_p(dpairs.data_ptr()), n, tol, max_level,
                                      ctypes.c_void_p(dJ.data_ptr()), ctypes.c_void_p(dP.data_ptr()),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, lib.i2_last_error().decode()
    torch.cuda.synchronize()
    return dJ.cpu().numpy(), dP.cpu().numpy()


def test_noalloc_matches_device_entry_point():
    torch = pytest.importorskip("torch")
    ensure_built()
    from integrator2_gb300 import _lib, api, meshes, pairs as P
    lib = _lib.lib()
    V, C = meshes.jittered_icosphere(3, 0.15, 7)
    far = P.build_pairs(V, C).far
    rng = np.random.default_rng(3)
    dV = torch.from_numpy(np.ascontiguousarray(V, np.float64)).cuda()
    dC = torch.from_numpy(np.ascontiguousarray(C, np.int32)).cuda()
    # two calls in a row with different pair lists, sizes and tolerances (the second finds the
    # first call's state in the shared scratch array)
    calls = [(far[np.sort(rng.choice(len(far), 12000, replace=False))], 1e-7, 5),
             (far[rng.choice(len(far), 5000, replace=False)][:, ::-1], 1e-9, 4)]
    for pairs, tol, lv in calls:
        J0, P0 = _existing(api, V, C, pairs, tol, lv)
        J1, P1 = _noalloc(lib, torch, dV, dC, pairs, tol, lv)
        assert np.isfinite(J1).all() and np.isfinite(P1).all()
        assert rel_rows(J1, J0).max() <= TOL
        assert (np.abs(P1 - P0) / np.abs(P0)).max() <= TOL

    # sizes beyond the static limits are rejected before any launch
    big = np.zeros((MAX_PAIRS + 1, 2), np.int32)
    dbig = torch.from_numpy(big).cuda()
    dJ = torch.zeros((MAX_PAIRS + 1, 3), dtype=torch.float64, device="cuda")
    dP = torch.zeros(MAX_PAIRS + 1, dtype=torch.float64, device="cuda")
    st = lib.i2_not_neighbors_noalloc(ctypes.c_void_p(dV.data_ptr()), dV.shape[0], ctypes.c_void_p(dC.data_ptr()),
                                      dC.shape[0], ctypes.c_void_p(dbig.data_ptr()), MAX_PAIRS + 1, 1e-7, 5,
                                      ctypes.c_void_p(dJ.data_ptr()), ctypes.c_void_p(dP.data_ptr()), None)
    assert st == I2_ERR_INVALID_ARGUMENT and "limit" in lib.i2_last_error().decode()
    st = lib.i2_not_neighbors_noalloc(ctypes.c_void_p(dV.data_ptr()), dV.shape[0], ctypes.c_void_p(dC.data_ptr()),
                                      MAX_CELLS + 1, ctypes.c_void_p(dbig.data_ptr()), 10, 1e-7, 5,
                                      ctypes.c_void_p(dJ.data_ptr()), ctypes.c_void_p(dP.data_ptr()), None)
    assert st == I2_ERR_INVALID_ARGUMENT
    assert torch.count_nonzero(dJ).item() == 0
