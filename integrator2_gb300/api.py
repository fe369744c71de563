"""Python mirror of the reference's host API (Mesh3D, QuadratureFormula3D, NumericalIntegrator3D,
EvaluatorJ3DK) over the C-ABI.  Method names and argument meaning follow the reference
(src/Mesh3d.cuh, src/NumericalIntegrator3d.cuh, src/evaluators/evaluator3d.cuh); results are
returned as numpy arrays at full precision instead of only through the text export.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib
from ._lib import call

SIMPLE_NEIGHBORS, ATTACHED_NEIGHBORS, NOT_NEIGHBORS, SELF = 0, 1, 2, 3
FIXED_REFINEMENT_LEVEL, AUTOMATIC_ERROR_CONTROL, RELATIVE_ERROR_CONTROL = 0, 1, 2
PRECISION_FP64, PRECISION_MIXED = 0, 1
PLAIN_TEXT, CSV, CSV_FULL_PRECISION = 0, 1, 2
_CH_J, _CH_P, _CH_RAW, _CH_ERR, _CH_LEVEL = 0, 1, 2, 3, 4


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def neighborTypeString(cls: int) -> str:
    """src/Mesh3d.cu:345-358"""
    return {0: "SimpleNeighbors", 1: "AttachedNeighbors", 2: "NotNeighbors", 3: "Self"}.get(cls, "")


@dataclass(frozen=True)
class QuadratureFormula3D:
    """Barycentric (L1, L2) coordinates, weights and Runge order (src/QuadratureFormula3d.cuh:20-31)."""
    coordinates: np.ndarray
    weights: np.ndarray
    order: int

    @staticmethod
    def builtin(npoints: int) -> "QuadratureFormula3D":
        c = np.zeros(2 * npoints)
        w = np.zeros(npoints)
        o = ctypes.c_int32()
        call("i2_quadrature_builtin", npoints, _p(c), _p(w), ctypes.byref(o))
        return QuadratureFormula3D(c.reshape(-1, 2), w, int(o.value))


# the reference's built-in rules, resolved by NumericalIntegrator3D (number of points)
qf3D1, qf3D3, qf3D4, qf3D6, qf3D7, qf3D9, qf3D12, qf3D13 = (1, 3, 4, 6, 7, 9, 12, 13)


class Mesh3D:
    """Surface mesh: vertices, cells, cell normals / measures and the pair lists."""

    def __init__(self):
        h = ctypes.c_void_p()
        call("i2_mesh_create", ctypes.byref(h))
        self._h = h
        self._lib = _lib.lib()

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.i2_mesh_destroy(self._h)
            self._h = None

    def loadMeshFromFile(self, filename: str, scale: float = 1.0) -> bool:
        """src/Mesh3d.cu:159-217; False (and a message in lastError()) if the file is unreadable."""
        code = self._lib.i2_mesh_load_file(self._h, filename.encode(), float(scale))
        return code == 0

    def setGeometry(self, vertices: np.ndarray, cells: np.ndarray) -> None:
        V = np.ascontiguousarray(vertices, np.float64).reshape(-1, 3)
        C = np.ascontiguousarray(cells, np.int32).reshape(-1, 3)
        call("i2_mesh_set_geometry", self._h, _p(V), len(V), _p(C), len(C))

    def prepareMesh(self, near_factor: Optional[float] = None) -> None:
        """src/Mesh3d.cu:219-226.  near_factor=None keeps every disjoint pair (the reference);
        a number keeps disjoint pairs closer than near_factor x mean edge length."""
        call("i2_mesh_prepare", self._h, float(near_factor) if near_factor else 0.0)

    def prepareMeshDevice(self, near_factor: Optional[float] = None, host_copy: bool = True) -> None:
        """prepareMesh with the pair lists built on the GPU (O(N), the same lists in the same
        order as prepareMesh).  host_copy=False keeps them on the device until a host-side call
        needs them; devicePairs() hands them out."""
        call("i2_mesh_prepare_device", self._h, float(near_factor) if near_factor else 0.0, 1 if host_copy else 0)

    def devicePairs(self, cls: int):
        """(device pointer, n) of a class's unordered int2 (i, j) rows, owned by the mesh."""
        ptr, n = ctypes.c_void_p(), ctypes.c_int64()
        call("i2_mesh_device_pairs", self._h, cls, ctypes.byref(ptr), ctypes.byref(n))
        return int(ptr.value or 0), int(n.value)

    def _count(self, cls: int) -> int:
        n = ctypes.c_int64()
        call("i2_mesh_pair_count", self._h, cls, ctypes.byref(n))
        return int(n.value)

    def _pairs(self, cls: int) -> np.ndarray:
        n = self._count(cls)
        rows = np.zeros((n, 3), np.int32)
        if n:
            call("i2_mesh_copy_pairs", self._h, cls, _p(rows), n)
        return rows

    def getSimpleNeighbors(self) -> np.ndarray:
        return self._pairs(SIMPLE_NEIGHBORS)

    def getAttachedNeighbors(self) -> np.ndarray:
        return self._pairs(ATTACHED_NEIGHBORS)

    def getNotNeighbors(self) -> np.ndarray:
        return self._pairs(NOT_NEIGHBORS)

    def getSelfPairs(self) -> np.ndarray:
        return self._pairs(SELF)

    def sizes(self):
        nv, nc = ctypes.c_int32(), ctypes.c_int32()
        call("i2_mesh_sizes", self._h, ctypes.byref(nv), ctypes.byref(nc))
        return int(nv.value), int(nc.value)

    def _cell_data(self):
        _, nc = self.sizes()
        n, s, c = np.zeros((nc, 3)), np.zeros(nc), np.zeros((nc, 3))
        call("i2_mesh_copy_cell_data", self._h, _p(n), _p(s), _p(c))
        return n, s, c

    def getCellNormals(self) -> np.ndarray:
        return self._cell_data()[0]

    def getCellMeasures(self) -> np.ndarray:
        return self._cell_data()[1]

    def getCellCenters(self) -> np.ndarray:
        return self._cell_data()[2]


class NumericalIntegrator3D:
    """Quadrature rule + refinement policy (src/NumericalIntegrator3d.cuh:73-327)."""

    def __init__(self, mesh: Mesh3D, qf):
        if isinstance(qf, int):
            qf = QuadratureFormula3D.builtin(qf)
        self.qf = qf
        c = np.ascontiguousarray(qf.coordinates, np.float64).reshape(-1)
        w = np.ascontiguousarray(qf.weights, np.float64)
        h = ctypes.c_void_p()
        call("i2_integrator_create", mesh._h, _p(c), _p(w), len(w), int(qf.order), ctypes.byref(h))
        self._h = h
        self._lib = _lib.lib()
        self.mesh = mesh

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.i2_integrator_destroy(self._h)
            self._h = None

    def setFixedRefinementLevel(self, refinementLevel: int = 0) -> None:
        call("i2_integrator_set_fixed_refinement_level", self._h, int(refinementLevel))

    def setErrorControl(self, mode: int, rel_tol: float = 1e-6, max_level: int = 5) -> None:
        call("i2_integrator_set_error_control", self._h, int(mode), float(rel_tol), int(max_level))

    def setPrecision(self, precision: int) -> None:
        call("i2_integrator_set_precision", self._h, int(precision))

    def setPotentialRule(self, n_radial=10, n_angular=8, grading=3, n_self=0) -> None:
        """graded Duffy rule of adjacent pairs; n_self points per edge piece of the self-pair edge
        rule (0: the closed form, exact, the default in both precisions)"""
        call("i2_integrator_set_potential_rule", self._h, n_radial, n_angular, grading, n_self)

    def setHardPairTolerance(self, rel_tol: float) -> None:
        """adaptive potential of folded / sliver adjacent pairs (0 disables)"""
        call("i2_integrator_set_hard_pair_tolerance", self._h, float(rel_tol))

    def setPotential(self, enabled: bool) -> None:
        """False: J only, as the reference computes it (the adjacent classes' potential rule is
        skipped and their P reads NaN)"""
        call("i2_integrator_set_potential", self._h, 1 if enabled else 0)

    def setSelfConvention(self, sign: int) -> None:
        call("i2_integrator_set_self_convention", self._h, int(sign))

    def getErrorControlType(self) -> int:
        m, lv = ctypes.c_int(), ctypes.c_int32()
        call("i2_integrator_get_error_control", self._h, ctypes.byref(m), ctypes.byref(lv))
        return int(m.value)

    def getGaussPointsNumber(self) -> int:
        return len(self.qf.weights)

    def getQuadratureFormulaOrder(self) -> int:
        return int(self.qf.order)


class EvaluatorJ3DK:
    """Pair integrals of the Newtonian kernel gradient and potential (src/evaluators/evaluatorJ3DK.cuh)."""

    def __init__(self, mesh: Mesh3D, numIntegrator: NumericalIntegrator3D):
        h = ctypes.c_void_p()
        call("i2_evaluator_create", mesh._h, numIntegrator._h, ctypes.byref(h))
        self._h = h
        self._lib = _lib.lib()
        self.mesh, self.integrator = mesh, numIntegrator

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.i2_evaluator_destroy(self._h)
            self._h = None

    def setStream(self, stream_handle: int) -> None:
        call("i2_evaluator_set_stream", self._h, ctypes.c_void_p(stream_handle))

    def runAllPairs(self, checkCorrectness: bool = False) -> None:
        call("i2_evaluator_run_all_pairs", self._h, int(bool(checkCorrectness)))

    def runPairs(self, simple, attached, notNeighbors) -> None:
        lists = [np.ascontiguousarray(np.asarray(l, np.int32).reshape(-1, 3)) for l in (simple, attached, notNeighbors)]
        call("i2_evaluator_run_pairs", self._h, _p(lists[0]), len(lists[0]), _p(lists[1]), len(lists[1]),
             _p(lists[2]), len(lists[2]))

    def runClass(self, cls: int, pairs) -> None:
        rows = np.ascontiguousarray(np.asarray(pairs, np.int32))
        stride = rows.shape[1] if rows.ndim == 2 else 2
        call("i2_evaluator_run_class", self._h, int(cls), _p(rows), len(rows), int(stride))

    def runClassDevice(self, cls: int, d_pairs_ptr: int, n: int, d_raw=0, d_J=0, d_P=0) -> None:
        """Hot path: device pointers (e.g. torch tensors' data_ptr()); asynchronous on the stream."""
        call("i2_evaluator_run_class_device", self._h, int(cls), ctypes.c_void_p(d_pairs_ptr), int(n),
             ctypes.c_void_p(d_raw or None), ctypes.c_void_p(d_J or None), ctypes.c_void_p(d_P or None))

    def backwardClass(self, cls: int, d_pairs_ptr: int, n: int, d_gJ=0, d_gP=0, d_gradV=0) -> None:
        """Adjoint of the last runClassDevice / runClass of this class (same pairs): adds
        gJ . dJ/dV + gP dP/dV to the device buffer d_gradV (3 doubles per vertex)."""
        call("i2_evaluator_backward_class", self._h, int(cls), ctypes.c_void_p(d_pairs_ptr), int(n),
             ctypes.c_void_p(d_gJ or None), ctypes.c_void_p(d_gP or None), ctypes.c_void_p(d_gradV))

    def getRunStats(self, cls: int) -> dict:
        """counters of the last run of a class (i2_evaluator_run_stats)"""
        out = np.zeros(15, np.int64)
        call("i2_evaluator_run_stats", self._h, cls, _p(out), len(out))
        return {"pairs": int(out[0]), "tier2": int(out[1]), "tier2b": int(out[2]), "adaptive_potential": int(out[3]),
                "adaptive_overflow": int(out[4]), "fp64_fixup": int(out[5]), "max_level": int(out[6]),
                "unconverged_after_level": [int(x) for x in out[7:14]], "fp64_fixup_spread": int(out[14])}

    def synchronize(self) -> None:
        call("i2_evaluator_synchronize", self._h)

    def resultCount(self, cls: int) -> int:
        n = ctypes.c_int64()
        call("i2_evaluator_result_count", self._h, int(cls), ctypes.byref(n))
        return int(n.value)

    def _channel(self, cls: int, ch: int, width: int) -> np.ndarray:
        n = self.resultCount(cls)
        out = np.zeros(n * width)
        if n:
            call("i2_evaluator_copy_results", self._h, int(cls), ch, _p(out), n)
        return out.reshape(n, width) if width > 1 else out

    def getResults(self, cls: int) -> np.ndarray:
        """J per pair, [n, 3] (the reference's d_*Results)."""
        return self._channel(cls, _CH_J, 3)

    def getIntegrals(self, cls: int) -> np.ndarray:
        """(Psi, Theta) per pair after the singular part, [n, 4] (the reference's d_*Integrals)."""
        return self._channel(cls, _CH_RAW, 4)

    def getPotentials(self, cls: int) -> np.ndarray:
        return self._channel(cls, _CH_P, 1)

    def getErrors(self, cls: int) -> np.ndarray:
        return self._channel(cls, _CH_ERR, 1)

    def getLevels(self, cls: int) -> np.ndarray:
        return self._channel(cls, _CH_LEVEL, 1).astype(np.int32)

    def outputResultsToFile(self, cls: int, outputFormat: int, path: Optional[str] = None) -> bool:
        """src/evaluators/evaluator3d.cu:354-457; default file name as in the reference."""
        if path is None:
            path = neighborTypeString(cls) + (".dat" if outputFormat == PLAIN_TEXT else ".csv")
        return self._lib.i2_evaluator_output_results(self._h, int(cls), int(outputFormat), path.encode()) == 0


class BatchEvaluator:
    """Batched form (no reference counterpart): many (mesh, pair class) segments integrated
    together by one persistent cooperative kernel per refinement sweep, captured in a CUDA graph
    on the first run and replayed afterwards.  Settings come from the integrator given here;
    the batch computes in mixed precision."""

    def __init__(self, numIntegrator: NumericalIntegrator3D):
        h = ctypes.c_void_p()
        call("i2_batch_create", numIntegrator._h, ctypes.byref(h))
        self._h = h
        self._lib = _lib.lib()
        self._keep = []  # meshes must outlive the batch
        self.integrator = numIntegrator

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.i2_batch_destroy(self._h)
            self._h = None

    def setStream(self, stream_handle: int) -> None:
        call("i2_batch_set_stream", self._h, ctypes.c_void_p(stream_handle))

    def add(self, mesh: Mesh3D, cls: int, pairs) -> int:
        rows = np.ascontiguousarray(np.asarray(pairs, np.int32))
        stride = rows.shape[1] if rows.ndim == 2 else 2
        seg = ctypes.c_int32()
        call("i2_batch_add", self._h, mesh._h, int(cls), _p(rows), len(rows), int(stride), ctypes.byref(seg))
        self._keep.append(mesh)
        return int(seg.value)

    def autotune(self):
        """times the candidate launch shapes; returns (threads, blocks per SM, lanes per pair,
        register variants as v_vertex + 3 v_edge + 9 v_disjoint)"""
        shape = np.zeros(4, np.int32)
        call("i2_batch_autotune", self._h, _p(shape))
        return tuple(int(x) for x in shape)

    def run(self) -> None:
        call("i2_batch_run", self._h)

    def usesGraph(self) -> bool:
        g = ctypes.c_int32()
        call("i2_batch_uses_graph", self._h, ctypes.byref(g))
        return bool(g.value)

    def resultCount(self, segment: int) -> int:
        n = ctypes.c_int64()
        call("i2_batch_result_count", self._h, int(segment), ctypes.byref(n))
        return int(n.value)

    def _channel(self, segment: int, ch: int, width: int) -> np.ndarray:
        n = self.resultCount(segment)
        out = np.zeros(n * width)
        if n:
            call("i2_batch_copy_results", self._h, int(segment), ch, _p(out), n)
        return out.reshape(n, width) if width > 1 else out

    def getResults(self, segment: int) -> np.ndarray:
        return self._channel(segment, _CH_J, 3)

    def getIntegrals(self, segment: int) -> np.ndarray:
        return self._channel(segment, _CH_RAW, 4)

    def getPotentials(self, segment: int) -> np.ndarray:
        return self._channel(segment, _CH_P, 1)

    def getLevels(self, segment: int) -> np.ndarray:
        return self._channel(segment, _CH_LEVEL, 1).astype(np.int32)


def lastError() -> str:
    return _lib.lib().i2_last_error().decode()
