"""The reference's own CUDA build on the GPU: a driver-API harness around
oracle/_ref/ref_kernels.cubin.  TEST INFRASTRUCTURE ONLY.

oracle/ref_cuda_build.sh compiles the reference's unmodified src/ (andreyypopov/integrator2)
for sm_103a into that cubin where the reference checkout exists; the cubin travels with the
repository to the GPU machine.  This module loads it into the current CUDA context (the one torch
uses) and launches the reference's OWN kernels in the order of its fixed-refinement host flow:

- mesh preparation: kCalculateCellNormal, kCalculateCellMeasure (src/Mesh3d.cu:23-71, 228-241);
- tasks (i, j, k) with k = row index, as runPairs builds them (src/evaluators/evaluator3d.cu:213-288);
- fixed level 0: refined mesh = original mesh, refined tasks = tasks
  (src/NumericalIntegrator3d.cu:232-276);
- fixed level 1: one refineMesh (kFillOrdinal, kSplitCell over every cell; :305-322, :400-420)
  and updateTasks (kCountOrCreateTasks counting, then creating; :500-558);
- numericalIntegration: kIntegrateRegularPart{Simple,Attached} / kIntegrateNotNeighbors over the
  refined tasks, integrals zeroed, gathered by kSumIntegrationResults
  (src/evaluators/evaluatorJ3DK.cu:893-960, src/NumericalIntegrator3d.cu:376-398);
- integrateOver*: kIntegrateSingularPart{Simple,Attached} added to the integrals, then
  kFinalizeSimpleNeighborsResults / kFinalizeNonSimpleResults (evaluatorJ3DK.cu:846-892).

Launch shapes are the reference's (256 threads, 1024 for kCountOrCreateTasks).  Buffers are torch
tensors; the quadrature tables go into the reference's __constant__ arrays as the
NumericalIntegrator3D constructor fills them (src/NumericalIntegrator3d.cu:196-214).  The
adaptive mode's host loop is not driven here (its results are pinned by the golden vectors made
from the reference's routines built for the host, tests/golden/).
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ref_kernels.cubin")
NAMES = os.path.join(HERE, "_ref", "ref_kernels.names")
THREADS, THREADS_MAX, MAX_GAUSS = 256, 1024, 13
VERTEX, EDGE, FAR = 0, 1, 2


def available() -> bool:
    return os.path.exists(CUBIN) and os.path.exists(NAMES)


def _short(mangled: str) -> str:
    m = re.match(r"_Z(\d+)", mangled)
    k = int(m.group(1))
    return mangled[m.end():m.end() + k]


class RefCuda:
    """the reference's kernels loaded into torch's CUDA context on the current device"""

    def __init__(self, qf=None):
        import torch
        from oracle import oracle as O
        self.torch = torch
        torch.zeros(1, device="cuda")  # torch's (primary) context is current on this thread from here on
        cu = ctypes.CDLL("libcuda.so.1")
        vp, u = ctypes.c_void_p, ctypes.c_uint
        cu.cuModuleLoad.argtypes = [ctypes.POINTER(vp), ctypes.c_char_p]
        cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(vp), vp, ctypes.c_char_p]
        cu.cuModuleGetGlobal_v2.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_size_t), vp, ctypes.c_char_p]
        cu.cuMemcpyHtoD_v2.argtypes = [ctypes.c_uint64, vp, ctypes.c_size_t]
        cu.cuLaunchKernel.argtypes = [vp, u, u, u, u, u, u, u, vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
        cu.cuModuleUnload.argtypes = [vp]
        self.cu = cu
        self.mod = vp()
        self._check(cu.cuModuleLoad(ctypes.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        self.fn = {}
        for mangled in open(NAMES).read().split():
            f = vp()
            self._check(cu.cuModuleGetFunction(ctypes.byref(f), self.mod, mangled.encode()), mangled)
            self.fn[_short(mangled)] = f
        coords, weights, _ = qf if qf is not None else O.QF13
        n = len(weights)
        L = np.zeros((n, 3))
        L[:, 0], L[:, 1] = coords[:, 0], coords[:, 1]
        L[:, 2] = 1.0 - coords[:, 0] - coords[:, 1]
        self._to_global("c_GaussPointsCoordinates", np.ascontiguousarray(L))
        self._to_global("c_GaussPointsWeights", np.ascontiguousarray(weights, np.float64))
        self._to_global("c_GaussPointsNumber", np.array([n], np.int32))
        self.npts = n

    def close(self):
        if self.mod:
            self.cu.cuModuleUnload(self.mod)
            self.mod = None

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"CUDA driver call failed ({what}): error {rc}")

    def _to_global(self, name, arr):
        ptr, size = ctypes.c_uint64(), ctypes.c_size_t()
        self._check(self.cu.cuModuleGetGlobal_v2(ctypes.byref(ptr), ctypes.byref(size), self.mod, name.encode()), name)
        if arr.nbytes > size.value:
            raise ValueError(f"{name}: {arr.nbytes} bytes into {size.value}")
        self._check(self.cu.cuMemcpyHtoD_v2(ptr.value, arr.ctypes.data_as(ctypes.c_void_p), arr.nbytes), name)

    def _launch(self, name, n, args, threads=THREADS):
        if n <= 0:
            return
        held = []
        for a in args:
            if isinstance(a, int):
                held.append(ctypes.c_int(a))
            elif a is None:
                held.append(ctypes.c_void_p(0))
            else:  # a torch tensor: its device pointer
                held.append(ctypes.c_void_p(a.data_ptr()))
        params = (ctypes.c_void_p * len(held))(*[ctypes.cast(ctypes.byref(h), ctypes.c_void_p) for h in held])
        stream = ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        blocks = (n + threads - 1) // threads
        self._check(self.cu.cuLaunchKernel(self.fn[name], blocks, 1, 1, threads, 1, 1, 0, stream, params, None), name)

    def prepare(self, V, C):
        """device mesh: vertices, cells, the reference's normals and measures"""
        t = self.torch
        m = {"V": t.as_tensor(np.ascontiguousarray(V, np.float64), device="cuda"),
             "C": t.as_tensor(np.ascontiguousarray(C, np.int32), device="cuda")}
        nc = len(C)
        m["N"] = t.empty(nc, 3, dtype=t.float64, device="cuda")
        m["S"] = t.empty(nc, dtype=t.float64, device="cuda")
        self._launch("kCalculateCellNormal", nc, [nc, m["V"], m["C"], m["N"]])
        self._launch("kCalculateCellMeasure", nc, [nc, m["V"], m["C"], m["S"]])
        return m

    def refine_once(self, m):
        """NumericalIntegrator3D::refineMesh with the whole mesh refined (fixed level 1)"""
        t = self.torch
        nv, nc = len(m["V"]), len(m["C"])
        temp_orig = t.empty(nc, dtype=t.int32, device="cuda")
        self._launch("kFillOrdinal", nc, [nc, temp_orig])
        rV = t.empty(nv + 3 * nc, 3, dtype=t.float64, device="cuda")
        rV[:nv] = m["V"]
        rC = t.empty(4 * nc, 3, dtype=t.int32, device="cuda")
        rS = t.empty(4 * nc, dtype=t.float64, device="cuda")
        orig = t.empty(4 * nc, dtype=t.int32, device="cuda")
        counts = t.tensor([nv, 0], dtype=t.int32, device="cuda")
        self._launch("kSplitCell", nc, [nc, rV, rC, rS, orig, counts, m["V"], m["C"], m["S"], temp_orig, None, None])
        return rV, rC, rS, orig, temp_orig

    def tasks(self, pairs):
        t = self.torch
        pairs = np.asarray(pairs, np.int32).reshape(-1, 2)
        tk = np.column_stack([pairs, np.arange(len(pairs), dtype=np.int32)]).astype(np.int32)
        return t.as_tensor(np.ascontiguousarray(tk), device="cuda")

    def setup_level(self, m, tasks, level):
        """(refined vertices, cells, measures, refined tasks) for a fixed refinement level 0 or 1"""
        if level == 0:
            return m["V"], m["C"], m["S"], tasks.clone()
        if level != 1:
            raise ValueError("the reference is self-consistent at fixed levels 0 and 1 only")
        t = self.torch
        rV, rC, rS, orig, temp_orig = self.refine_once(m)
        n, ncr = len(tasks), len(rC)
        cnt = t.zeros(1, dtype=t.int32, device="cuda")
        self._launch("kCountOrCreateTasks", n, [n, ncr, cnt, tasks, orig, temp_orig, None, None, None], THREADS_MAX)
        k = int(cnt.item())
        rt = t.empty(k, 3, dtype=t.int32, device="cuda")
        cnt.zero_()
        self._launch("kCountOrCreateTasks", n, [n, ncr, cnt, tasks, orig, temp_orig, None, None, rt], THREADS_MAX)
        return rV, rC, rS, rt

    def integrate(self, cls, m, tasks, refined, integrals, results, J):
        """numericalIntegration + integrateOver* of one class: regular part over the refined
        tasks, gather, singular part, finalisation (J into J)"""
        rV, rC, rS, rt = refined
        n, k = len(tasks), len(rt)
        if cls == VERTEX:
            self._launch("kIntegrateRegularPartSimple", k, [k, results, rt, tasks, m["V"], m["C"], m["N"], m["S"], rV, rC, rS, self.npts])
        elif cls == EDGE:
            self._launch("kIntegrateRegularPartAttached", k, [k, results, rt, tasks, m["V"], m["C"], m["N"], rV, rC, rS, self.npts])
        else:
            self._launch("kIntegrateNotNeighbors", k, [k, results, rt, m["V"], m["C"], rV, rC, rS, self.npts])
        integrals.zero_()
        self._launch("kSumIntegrationResults", k, [k, integrals, results, rt])
        if cls == VERTEX:
            self._launch("kIntegrateSingularPartSimple", n, [n, integrals, tasks, m["V"], m["C"], m["N"], m["S"]])
            self._launch("kFinalizeSimpleNeighborsResults", n, [n, J, integrals, tasks, m["N"], m["S"]])
        elif cls == EDGE:
            self._launch("kIntegrateSingularPartAttached", n, [n, integrals, tasks, m["V"], m["C"], m["N"], m["S"]])
            self._launch("kFinalizeNonSimpleResults", n, [n, J, integrals, tasks, m["N"]])
        else:
            self._launch("kFinalizeNonSimpleResults", n, [n, J, integrals, tasks, m["N"]])

    def run(self, cls, V, C, pairs, level=0):
        """the reference's (Psi, Theta) integrals [n, 4] and J [n, 3] for ordered pairs of one
        class at a fixed refinement level (0 or 1)"""
        t = self.torch
        m = self.prepare(V, C)
        tasks = self.tasks(pairs)
        refined = self.setup_level(m, tasks, level)
        n = len(tasks)
        integrals = t.zeros(n, 4, dtype=t.float64, device="cuda")
        results = t.empty(len(refined[3]), 4, dtype=t.float64, device="cuda")
        J = t.empty(n, 3, dtype=t.float64, device="cuda")
        self.integrate(cls, m, tasks, refined, integrals, results, J)
        t.cuda.synchronize()
        return integrals.cpu().numpy(), J.cpu().numpy()

    def time_class(self, cls, V, C, pairs, level=0, steps=5, warmup=2):
        """device time in ms of integrateOver<class> (the reference's own GpuTimer bracket,
        evaluator3d.cu:173-186: regular part, gather, singular part, finalisation), mean of
        `steps` runs with the tasks and refined mesh already on the device"""
        t = self.torch
        m = self.prepare(V, C)
        tasks = self.tasks(pairs)
        refined = self.setup_level(m, tasks, level)
        n = len(tasks)
        integrals = t.zeros(n, 4, dtype=t.float64, device="cuda")
        results = t.empty(len(refined[3]), 4, dtype=t.float64, device="cuda")
        J = t.empty(n, 3, dtype=t.float64, device="cuda")
        for _ in range(warmup):
            self.integrate(cls, m, tasks, refined, integrals, results, J)
        t.cuda.synchronize()
        e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            self.integrate(cls, m, tasks, refined, integrals, results, J)
        e1.record()
        t.cuda.synchronize()
        return e0.elapsed_time(e1) / steps
