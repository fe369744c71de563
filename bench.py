"""Benchmark of the pair-integral path on one GB300.

Workload (one "step"): every ordered pair of the four pair classes of a 20,480-triangle
icosphere (5 subdivisions) whose vertices carry a seeded tangential Gaussian jitter of 0.15 x
mean edge length, reprojected to the unit sphere: common-vertex, common-edge, self, and
disjoint pairs with centroid distance < 3 x mean edge length (1,418,734 ordered pairs), each
producing J (3-vector) and P.  Refinement: relative error control (|J_L - J_{L-1}| <= tol |J_L|,
levels 0..5) with the 13-point degree-7 rule; the potential of adjacent pairs uses the graded
Duffy rule.  Data are synthetic (no data set exists for this path).

value  = pair-integrals/s with pair lists and outputs resident in HBM (CUDA events on the
         launching stream, L2 flushed between steps by a 512 MiB write).
e2e    = the same through the C-ABI from pinned host lists: H2D of the lists and D2H of J and P
         inside the timed region.
roofline: the pair kernels are bounded by the FP32 pipe (mixed bulk: `roofline`) or the FP64 pipe
         (plain form: `roofline_fp64`); peaks are measured live by i2_calibrate_pipes
         (MEASURED_PEAKS.json carries only HBM and bf16 figures).
cpu_baseline: the oracle (a C restatement of the reference's formulas, OpenMP) on the host, over
         every pair of the workload.  --impl reference times the same over every pair in each of
         its timed steps.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CLASSES = (0, 1, 2, 3)  # vertex, edge, near-field, self
SEED = 2026
NEAR = 3.0


# ------------------------------------------------------------------ workload
def workload():
    from integrator2_gb300 import meshes, pairs
    V, C = meshes.jittered_icosphere(5, 0.15, SEED)
    pl = pairs.build_pairs(V, C, NEAR)
    return V, C, {c: np.ascontiguousarray(pl.by_class(c)) for c in CLASSES}


# ------------------------------------------------------------------ algorithmic work model
# Frozen per-integrand-evaluation operation counts of the restated formulas (FP64):
# (arithmetic flops, sqrt, divide, log, atan2).  Far: theta/psi + potential (a1 + a18);
# edge / vertex: fused regular part (a1 - a2 / a1 - a3); duffy: inner potential per Duffy
# point; closed forms (a4 / a5) per adjacent pair: (flops, sqrt, div, log, atan2, sincos, acos).
POINT_OPS = {"far": (160, 3, 3, 3, 1), "edge": (175, 3, 0, 2, 3), "vertex": (185, 3, 1, 3, 3),
             "duffy": (175, 3, 3, 3, 1)}
CLOSED_OPS = {"edge": (260, 0, 14, 11, 4, 5, 4), "vertex": (420, 0, 22, 14, 10, 12, 3)}


def flop_weights(cal):
    """flop equivalents (2 per FMA time unit) of sqrt, div, log, atan2, sincos, acos"""
    return {k: 2.0 * cal[2 + i] for i, k in enumerate(("sqrt", "div", "log", "atan2", "sincos", "acos"))}


def point_flops(kind, w):
    a, s, d, l, t = POINT_OPS[kind]
    return a + s * w["sqrt"] + d * w["div"] + l * w["log"] + t * w["atan2"]


def closed_flops(kind, w):
    a, s, d, l, t, sc, ac = CLOSED_OPS[kind]
    return a + s * w["sqrt"] + d * w["div"] + l * w["log"] + t * w["atan2"] + sc * w["sincos"] + ac * w["acos"]


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", "0", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU leg
def cpu_run(V, C, lists, frac, tol, nthreads=0):
    """the oracle with the product's rules on every pair of every class (frac >= 1) or on a
    seeded sample (fraction frac of every class); returns (pairs, seconds, threads)"""
    from oracle import oracle as O
    rng = np.random.default_rng(1)
    n = 0
    with O.potential_rule(**O.PRODUCT_RULE):
        t0 = time.perf_counter()
        for cls in CLASSES:
            pr = lists[cls]
            if frac < 1.0:
                pr = pr[np.sort(rng.choice(len(pr), max(1, int(len(pr) * frac)), replace=False))]
            O.integrate(cls, pr, V, C, mode=O.ADAPTIVE_RELATIVE, tol=tol, nthreads=nthreads)
            n += len(pr)
        dt = time.perf_counter() - t0
    return n, dt, (nthreads or O.lib().o_max_threads())


def workload_config(total, tol):
    """the config dict both arms print (the same workload, rules and error control)"""
    return {"workload": "jittered icosphere s5 (20480 triangles, sigma 0.15h, seed 2026): common-vertex, "
                        "common-edge, self and near-field (< 3h) ordered pairs",
            "pairs": int(total), "error_control": f"relative tol {tol}, levels 0..5",
            "rule": "qf3D13; adjacent potential: tiered graded Duffy 10x8 / 8x6 check / 16x16 / adaptive"}


def level0_workloads():
    """C1 (icosphere s2, 320 triangles) and the C2 workload: the pair lists of the reference's
    three classes, for the J-only fixed-level-0 comparison with the reference's CUDA build"""
    from integrator2_gb300 import meshes, pairs
    V1, C1 = meshes.icosphere(2)
    pl = pairs.build_pairs(V1, C1, NEAR)
    V2, C2, l2 = workload()
    return {"C1": (V1, C1, {c: pl.by_class(c) for c in (0, 1, 2)}), "C2": (V2, C2, {c: l2[c] for c in (0, 1, 2)})}


def reference_cuda_section():
    """the reference's own CUDA build (its src/ compiled unmodified for sm_103a, a cubin built
    where the reference checkout exists) on this GPU: integrateOver<class> timed per class as the
    reference's GpuTimer brackets it (regular part, gather, singular part, finalisation), fixed
    refinement level 0, qf3D13, J only (the reference computes no potential)"""
    try:
        from oracle import ref_cuda
        if not ref_cuda.available():
            return {"unavailable": "oracle/_ref/ref_kernels.cubin was not built (the reference checkout is needed where it is built)"}
        ref = ref_cuda.RefCuda()
    except Exception as e:  # no GPU or no driver
        return {"unavailable": f"{type(e).__name__}: {e}"}
    out = {}
    for name, (V, C, lists) in level0_workloads().items():
        ms = {CLASS_NAMES[c]: ref.time_class(c, V, C, lists[c], 0) for c in (0, 1, 2)}
        n = sum(len(lists[c]) for c in (0, 1, 2))
        out[name] = {"pairs": int(n), "class_ms": ms, "ms_per_step": float(sum(ms.values())),
                     "value": n / (sum(ms.values()) * 1e-3), "unit": "pair-integrals/s (J only, fixed level 0)"}
    ref.close()
    return out


def reference_arm(args):
    """the reference's formulas on the host cores: the oracle (a C restatement of the reference's
    path, OpenMP over pairs, the product's rules) over EVERY pair of the workload in each timed
    step; warm-up steps run a 1 % sample"""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    V, C, lists = workload()
    total = sum(len(v) for v in lists.values())
    for _ in range(args.warmup):
        cpu_run(V, C, lists, 0.01, args.tol)
    times, threads = [], 1
    for _ in range(args.steps):
        n, dt, threads = cpu_run(V, C, lists, 1.0, args.tol)
        assert n == total
        times.append(dt)
    ms = 1e3 * float(np.sum(times)) / args.steps
    v = total / (ms * 1e-3)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "pair-integrals/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(total, args.tol),
            "form": "the reference's formulas (oracle C restatement, FP64) on the host cores, OpenMP over pairs",
            "cpu_baseline": {"value": v, "unit": "pair-integrals/s", "cores": threads, "kind": "port",
                             "sample": f"every pair of the workload ({total} pairs) in each of {args.steps} timed steps"},
            "e2e": {"value": v, "unit": "pair-integrals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if "level0" in args.sections:
        line["reference_cuda"] = reference_cuda_section()
    print(json.dumps(line))


# "<= 1e-6" holds per pair at the 99.9th percentile and normwise; about 0.06 % of the pairs (FP32
# rounding of the edge logs amplified by the cancellation in Psi) lie above it, up to ~5e-6: the
# line's accuracy_statement gives the measured figures over every pair
METRIC = "pair-integrals/s at <=1e-6 rel err (per pair at p99.9 and normwise; tail share in accuracy_statement)"


# ------------------------------------------------------------------ GPU arm
CLASS_NAMES = {0: "vertex", 1: "edge", 2: "near", 3: "self"}


def class_accuracy(V, C, cls, pr, j, p):
    """relative error of one class's sampled rows pr (results j, p) against the oracle's
    high-order answer (fixed level 4 of the 13-point rule for J; for the potential of adjacent
    pairs the adaptive rule at 1e-10 on every pair): the largest per-pair error, its 99th
    percentile and rms, and the normwise error |dJ| / |J| over the sample"""
    from oracle import oracle as O
    with O.potential_rule(40, 32, 3, adaptive=1e-10, depth=18, every_pair=True):
        _, oJ, oP, _ = O.integrate(cls, pr, V, C, mode=O.FIXED, level=4 if cls != 3 else 0)
    if cls == 3:
        return {"J_abs_max": float(np.abs(j - oJ).max()), "P": float((np.abs(p - oP) / np.abs(oP)).max()), "sample": int(len(pr))}
    eJ = np.linalg.norm(j - oJ, axis=1) / np.maximum(np.linalg.norm(oJ, axis=1), 1e-300)
    eP = np.abs(p - oP) / np.abs(oP)
    return {"J": float(eJ.max()), "P": float(eP.max()),
            "J_p99": float(np.percentile(eJ, 99)), "P_p99": float(np.percentile(eP, 99)),
            "J_rms": float(np.sqrt(np.mean(eJ ** 2))), "P_rms": float(np.sqrt(np.mean(eP ** 2))),
            "J_normwise": float(np.linalg.norm(j - oJ) / np.linalg.norm(oJ)),
            "P_normwise": float(np.linalg.norm(p - oP) / np.linalg.norm(oP)), "sample": int(len(pr))}


def accuracy(V, C, lists, J, P, levels, nsample=400):
    """class_accuracy on a seeded sample of every class"""
    rng = np.random.default_rng(5)
    out = {}
    for cls in CLASSES:
        pr = lists[cls]
        idx = np.sort(rng.choice(len(pr), min(nsample, len(pr)), replace=False))
        out[CLASS_NAMES[cls]] = class_accuracy(V, C, cls, pr[idx], J[cls][idx], P[cls][idx])
    return out


def example_surfaces_section():
    """the mixed form against the FP64 form on the reference's example surfaces at the scales its
    README gives (the meshes and 800 seeded pairs per class each from tests/golden/examples.npz;
    relative control 1e-6): per class the 99th percentile and the maximum of the per-pair relative
    error of J and P.  The first three are well-conditioned; Girja, Fish and s5m hold pairs whose
    sensitivity to relative coordinate perturbations runs into the thousands, where FP32 point
    positions limit the mixed form to about that sensitivity x 1e-8."""
    from integrator2_gb300 import api
    d = np.load(os.path.join(ROOT, "tests", "golden", "examples.npz"))
    out = {}
    for mesh in ("G1", "Krylo01", "ellipsoid2000", "Girja", "Fish", "s5m"):
        V, C = d[f"{mesh}|V"], d[f"{mesh}|C"]
        row = {}
        for cls, name in ((0, "vertex"), (1, "edge"), (2, "near")):
            pr = np.ascontiguousarray(d[f"{mesh}|pairs_{cls}"])
            res = {}
            for prec in (api.PRECISION_FP64, api.PRECISION_MIXED):
                m = api.Mesh3D()
                m.setGeometry(V, C)
                m.prepareMesh(NEAR)
                it = api.NumericalIntegrator3D(m, api.qf3D13)
                it.setErrorControl(api.RELATIVE_ERROR_CONTROL, 1e-6, 5)
                it.setPrecision(prec)
                ev = api.EvaluatorJ3DK(m, it)
                ev.runClass(cls, pr)
                res[prec] = (ev.getResults(cls), ev.getPotentials(cls))
            (J64, P64), (Jm, Pm) = res[api.PRECISION_FP64], res[api.PRECISION_MIXED]
            eJ = np.linalg.norm(Jm - J64, axis=1) / np.linalg.norm(J64, axis=1)
            eP = np.abs(Pm - P64) / np.abs(P64)
            row[name] = {"pairs": int(len(pr)), "J_p99": float(np.percentile(eJ, 99)), "J_max": float(eJ.max()),
                         "P_p99": float(np.percentile(eP, 99)), "P_max": float(eP.max())}
        out[mesh] = row
    return {"vs": "FP64 form, relative control 1e-6", "scales": {"Fish": 100.0, "s5m": 0.0005}, "meshes": out}


def level0_j_only(stream, precision):
    """the library on the reference's own workload: J only (potential off), fixed refinement
    level 0, qf3D13, the reference's three classes on C1 and C2, per class through the device
    entry point (lists resident), CUDA events, mean of 5 runs after 2"""
    import torch
    from integrator2_gb300 import api
    out = {}
    for name, (V, C, lists) in level0_workloads().items():
        m = api.Mesh3D()
        m.setGeometry(V, C)
        m.prepareMesh(NEAR)
        it = api.NumericalIntegrator3D(m, api.qf3D13)
        it.setFixedRefinementLevel(0)
        it.setPotential(False)
        it.setPrecision(precision)
        ev = api.EvaluatorJ3DK(m, it)
        ev.setStream(stream.cuda_stream)
        ms = {}
        with torch.cuda.stream(stream):
            for c in (0, 1, 2):
                d = torch.from_numpy(np.ascontiguousarray(lists[c])).cuda()
                J = torch.empty(len(d), 3, dtype=torch.float64, device="cuda")
                P = torch.empty(len(d), dtype=torch.float64, device="cuda")
                for _ in range(2):
                    ev.runClassDevice(c, d.data_ptr(), len(d), 0, J.data_ptr(), P.data_ptr())
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(5):
                    ev.runClassDevice(c, d.data_ptr(), len(d), 0, J.data_ptr(), P.data_ptr())
                e1.record(stream)
                torch.cuda.synchronize()
                ms[CLASS_NAMES[c]] = e0.elapsed_time(e1) / 5
        n = sum(len(lists[c]) for c in (0, 1, 2))
        out[name] = {"pairs": int(n), "class_ms": ms, "ms_per_step": float(sum(ms.values())),
                     "value": n / (sum(ms.values()) * 1e-3), "unit": "pair-integrals/s (J only, fixed level 0)"}
    return out


def full_population(lists, form, fp64):
    """the form against the FP64 form on EVERY pair of the workload, per class and channel: the
    count and share of pairs above 1e-6 relative, the largest error, p99.9 and the pairs where the
    two forms kept different refinement levels"""
    out = {}
    for cls in CLASSES:
        j, j64 = form["J"][cls], fp64["J"][cls]
        p, p64 = form["P"][cls], fp64["P"][cls]
        if cls == 3:
            eJ = np.abs(j - j64).max(axis=1) / max(np.abs(j64).max(), 1e-300)
        else:
            eJ = np.linalg.norm(j - j64, axis=1) / np.maximum(np.linalg.norm(j64, axis=1), 1e-300)
        eP = np.abs(p - p64) / np.maximum(np.abs(p64), 1e-300)
        d = {"pairs": int(len(j))}
        for ch, e in (("J", eJ), ("P", eP)):
            d[ch] = {"above_1e-6": int(np.sum(e > 1e-6)), "share_above_1e-6": float(np.mean(e > 1e-6)),
                     "max": float(e.max()), "p99.9": float(np.percentile(e, 99.9)), "p99": float(np.percentile(e, 99))}
        if cls != 3:
            d["levels_differ"] = int(np.sum(form["levels"][cls] != fp64["levels"][cls]))
        out[CLASS_NAMES[cls]] = d
    return out


def accuracy_statement(pop, sampled):
    """one sentence with the measured per-pair figures behind the metric's "<= 1e-6" """
    if not pop:
        return None
    cls = [c for c in ("vertex", "edge", "near") if c in pop]
    n = sum(pop[c]["pairs"] for c in cls)
    above = {ch: sum(pop[c][ch]["above_1e-6"] for c in cls) for ch in ("J", "P")}
    p999 = {ch: max(pop[c][ch]["p99.9"] for c in cls) for ch in ("J", "P")}
    mx = {ch: max(pop[c][ch]["max"] for c in cls) for ch in ("J", "P")}
    nw = max(sampled[c]["J_normwise"] for c in cls) if sampled else None
    return (f"against the FP64 form over all {n} non-self pairs: per-pair p99.9 {p999['J']:.2e} (J) / {p999['P']:.2e} (P); "
            f"{above['J']} (J) and {above['P']} (P) pairs above 1e-6 ({100 * above['J'] / n:.3f} % / {100 * above['P'] / n:.3f} %), "
            f"max {mx['J']:.2e} / {mx['P']:.2e}; self pairs exact; normwise vs the high-order oracle {nw:.1e} (J, sampled)")


class DeviceRows:
    """a device int32 [n, 2] array owned by the library, seen by torch without a copy"""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n, 2), "typestr": "<i4", "data": (ptr, False), "version": 3}


def c5_section(args):
    """C5: torus R = 1, r = 0.1 on a 2000 x 500 grid (2 M triangles), scaled by 5e-4, normal jitter
    0.05 x the local edge length (seed 2026).  The pair lists are built on the GPU
    (i2_mesh_prepare_device; the host builder is timed beside it and must give the same lists),
    then all four classes (near < 3h, ordered pairs) run in mixed precision with relative error
    control 1e-6 through the device entry point, lists and results resident on the device: one
    warm-up step, two timed steps, CUDA events.  Accuracy: 200 sampled pairs per class against the
    oracle on the same geometry scaled by 2^20 (exact integrals scale as s^2 for J and s^3 for P;
    at that scale the oracle's absolute thresholds are in their normal range)."""
    import torch
    from integrator2_gb300 import api, meshes
    V, C = meshes.torus(2000, 500, 1.0, 0.1, scale=5e-4, jitter_rel=0.05, seed=SEED)
    e = np.linalg.norm(V[C[:, [1, 2, 0]]] - V[C], axis=2)
    aspect = e.max(axis=1) / e.min(axis=1)
    m = api.Mesh3D()
    m.setGeometry(V, C)
    m.prepareMeshDevice(NEAR, host_copy=False)  # first call: allocations and module loading
    t0 = time.perf_counter()
    m.prepareMeshDevice(NEAR, host_copy=False)
    t_dev = time.perf_counter() - t0
    h = api.Mesh3D()
    h.setGeometry(V, C)
    t0 = time.perf_counter()
    h.prepareMesh(NEAR)
    t_host = time.perf_counter() - t0
    rows, counts = {}, {}
    for c in CLASSES:
        ptr, n = m.devicePairs(c)
        u = torch.as_tensor(DeviceRows(ptr, n), device="cuda")
        if c != 3:
            hp, hn = h.devicePairs(c)
            if hn != n or not torch.equal(u, torch.as_tensor(DeviceRows(hp, hn), device="cuda")):
                raise RuntimeError(f"C5: device and host pair builders disagree on class {c}")
        rows[c] = u if c == 3 else torch.cat([u, u.flip(1)]).contiguous()
        counts[CLASS_NAMES[c]] = int(len(rows[c]))
    del h
    total = sum(counts.values())
    it = api.NumericalIntegrator3D(m, api.qf3D13)
    it.setErrorControl(api.RELATIVE_ERROR_CONTROL, args.tol, 5)
    it.setPrecision(api.PRECISION_MIXED)
    stream = torch.cuda.Stream()
    ev = api.EvaluatorJ3DK(m, it)
    ev.setStream(stream.cuda_stream)
    J = {c: torch.empty(len(rows[c]), 3, dtype=torch.float64, device="cuda") for c in CLASSES}
    P = {c: torch.empty(len(rows[c]), dtype=torch.float64, device="cuda") for c in CLASSES}
    torch.cuda.synchronize()  # the rows were made on torch's default stream; the evaluator runs on `stream`

    def step():
        for c in CLASSES:
            ev.runClassDevice(c, rows[c].data_ptr(), len(rows[c]), 0, J[c].data_ptr(), P[c].data_ptr())

    steps = 2
    with torch.cuda.stream(stream):
        step()
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler() as clk:
            e0.record(stream)
            for _ in range(steps):
                step()
            e1.record(stream)
            torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    rng = np.random.default_rng(7)
    acc = {}
    s = 2.0 ** 20
    for c in CLASSES:
        idx = torch.as_tensor(np.sort(rng.choice(len(rows[c]), 200, replace=False)), device="cuda")
        pr = rows[c][idx].cpu().numpy()
        acc[CLASS_NAMES[c]] = class_accuracy(V * s, C, c, pr, J[c][idx].cpu().numpy() * s ** 2, P[c][idx].cpu().numpy() * s ** 3)
    backward = c5_backward(V, C, rows, ev, stream, args.c5_backward_fraction)
    return {"workload": "C5: torus R=1, r=0.1, 2000 x 500 grid, x 5e-4, normal jitter 0.05 h, near < 3h, relative 1e-6, mixed",
            "triangles": int(len(C)), "pairs": int(total), "pairs_by_class": counts, "backward": backward,
            "edge_length": [float(e.min()), float(e.max())], "aspect_ratio": {"mean": float(aspect.mean()), "max": float(aspect.max())},
            "pair_builder_s": {"gpu": t_dev, "host": t_host, "same_lists": True},
            "value": total / (ms * 1e-3), "unit": "pair-integrals/s", "ms_per_step": ms, "steps": steps, "warmup": 1,
            "clocks": clk.summary(), "accuracy": acc}


def c5_backward(V, C, all_rows, ev, stream, fraction, ncoords=3):
    """adjoint of L = sum_p (gJ_p . J_p + gP_p P_p) (seeded gJ, gP ~ N(0, 1)) after the mixed C5
    forward pass, on a seeded share `fraction` of every class's pairs (1: all 194 M pairs; the
    adjacent classes' adjoint recomputes their rules in FP64 dual numbers, which makes a full pass
    take minutes): the forward pass over the sample, then the FP32 adjoint with the refined
    sub-cells recomputed at the levels the forward kept (one timed pass, CUDA events); spot check
    on a few coordinates against central differences of the FP64 forward with every sampled pair
    held at its kept level (h = 1e-6 x the local edge length), each over the sampled pairs that
    touch the coordinate's vertex, run on the sub-mesh of the cells those pairs use (a pair's
    integrals depend on its two cells only)"""
    import torch
    from integrator2_gb300 import api
    gen = torch.Generator(device="cuda").manual_seed(3)
    rows = {}
    # everything the evaluator reads is made on the evaluator's stream and finished before its
    # launches (the evaluator runs on `stream`, not on torch's default stream)
    with torch.cuda.stream(stream):
        for c in CLASSES:
            n = len(all_rows[c])
            k = n if fraction >= 1 else max(1, int(n * fraction))
            sel = torch.randperm(n, device="cuda", generator=gen)[:k].sort().values if k < n else None
            rows[c] = all_rows[c] if sel is None else all_rows[c][sel].contiguous()
        gJ = {c: torch.randn(len(rows[c]), 3, dtype=torch.float64, device="cuda", generator=gen) for c in CLASSES}
        gP = {c: torch.randn(len(rows[c]), dtype=torch.float64, device="cuda", generator=gen) for c in CLASSES}
        gradV = torch.zeros(len(V), 3, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for c in CLASSES:
            if len(rows[c]) < len(all_rows[c]):  # the forward pass over the sample (backward needs it just before)
                k = len(rows[c])
                J = torch.empty(k, 3, dtype=torch.float64, device="cuda")
                P = torch.empty(k, dtype=torch.float64, device="cuda")
                ev.runClassDevice(c, rows[c].data_ptr(), k, 0, J.data_ptr(), P.data_ptr())
        torch.cuda.synchronize()
    cls_ms = {}
    with torch.cuda.stream(stream):
        torch.cuda.synchronize()
        for c in CLASSES:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ev.backwardClass(c, rows[c].data_ptr(), len(rows[c]), gJ[c].data_ptr(), gP[c].data_ptr(), gradV.data_ptr())
            e1.record(stream)
            torch.cuda.synchronize()
            cls_ms[CLASS_NAMES[c]] = e0.elapsed_time(e1)
    ms = sum(cls_ms.values())
    g = gradV.cpu().numpy().reshape(-1)
    levels = {c: torch.as_tensor(ev.getLevels(c), device="cuda") if c != 3 else torch.zeros(len(rows[c]), dtype=torch.int32, device="cuda")
              for c in CLASSES}
    rng = np.random.default_rng(9)
    Ct = torch.as_tensor(np.asarray(C, np.int32), device="cuda")
    checks = []
    for k in rng.choice(V.size, ncoords, replace=False):
        v = int(k) // 3
        cells = torch.nonzero((Ct == v).any(dim=1)).flatten()
        edge = float(np.linalg.norm(V[C[int(cells[0])]][1] - V[C[int(cells[0])]][0]))
        h = 1e-6 * edge
        sub = {}
        for c in CLASSES:
            m = torch.isin(rows[c][:, 0], cells) | torch.isin(rows[c][:, 1], cells)
            sub[c] = (rows[c][m].cpu().numpy(), levels[c][m].cpu().numpy(), gJ[c][m].cpu().numpy(), gP[c][m].cpu().numpy())
        used = np.unique(np.concatenate([sub[c][0].reshape(-1) for c in CLASSES]))
        Cs = np.asarray(C)[used]
        vused, Cl = np.unique(Cs.reshape(-1), return_inverse=True)
        Cl = Cl.reshape(-1, 3).astype(np.int32)
        remap = {int(x): i for i, x in enumerate(used)}
        vals = []
        for sgn in (1.0, -1.0):
            Vp = np.array(V, np.float64)
            Vp.reshape(-1)[k] += sgn * h
            m = api.Mesh3D()
            m.setGeometry(np.ascontiguousarray(Vp[vused]), Cl)
            m.prepareMesh(NEAR)
            tot = 0.0
            for c in CLASSES:
                pr, lev, gj, gp = sub[c]
                if not len(pr):
                    continue
                prl = np.vectorize(remap.get)(pr).astype(np.int32).reshape(-1, 2)
                for L in np.unique(lev):
                    sel = lev == L
                    it = api.NumericalIntegrator3D(m, api.qf3D13)
                    it.setFixedRefinementLevel(int(max(L, 0)))
                    e = api.EvaluatorJ3DK(m, it)
                    e.runClass(c, prl[sel])
                    tot += float(np.sum(gj[sel] * e.getResults(c)) + np.sum(gp[sel] * e.getPotentials(c)))
            vals.append(tot)
        fd = (vals[0] - vals[1]) / (2 * h)
        checks.append({"coordinate": int(k), "adjoint": float(g[k]), "fd": fd, "abs_err_over_max_grad": abs(fd - g[k]) / np.abs(g).max()})
    npairs = int(sum(len(rows[c]) for c in CLASSES))
    return {"ms": ms, "class_ms": cls_ms, "pairs": npairs, "pairs_per_s": npairs / (ms * 1e-3),
            "sample": "every pair" if fraction >= 1 else f"seeded {fraction:.0%} of every class ({npairs} pairs)",
            "variant": "FP32 adjoint (after the mixed forward), sub-cells recomputed at the kept levels",
            "fd_spot_check": {"coordinates": checks, "of": "FP64 forward at the kept levels", "h": "1e-6 x local edge length",
                              "max_abs_err_over_max_grad": max(x["abs_err_over_max_grad"] for x in checks)}}


def run_form(ev, lists, d_pairs, d_J, d_P, stream, flush, steps, warmup):
    """times `steps` device-resident steps (L2 flushed between steps); returns the total device
    time in ms and the mean per-class time"""
    import torch
    with torch.cuda.stream(stream):
        for _ in range(max(warmup, 3)):
            for c in CLASSES:
                ev.runClassDevice(c, d_pairs[c].data_ptr(), len(lists[c]), 0, d_J[c].data_ptr(), d_P[c].data_ptr())
        stream.synchronize()
        ev_start = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ev_cls = [[torch.cuda.Event(enable_timing=True) for _ in CLASSES] for _ in range(steps)]
        for s in range(steps):
            flush.fill_(float(s))
            ev_start[s].record(stream)
            for k, c in enumerate(CLASSES):
                ev.runClassDevice(c, d_pairs[c].data_ptr(), len(lists[c]), 0, d_J[c].data_ptr(), d_P[c].data_ptr())
                ev_cls[s][k].record(stream)
        torch.cuda.synchronize()
    total = sum(ev_start[s].elapsed_time(ev_cls[s][-1]) for s in range(steps))
    cls_ms = np.zeros(len(CLASSES))
    for s in range(steps):
        prev = ev_start[s]
        for k in range(len(CLASSES)):
            cls_ms[k] += prev.elapsed_time(ev_cls[s][k])
            prev = ev_cls[s][k]
    return total, cls_ms / steps


def run_batch(batch, flush, stream, steps, warmup):
    """times `steps` replays of the batched form (CUDA graph of the whole step; L2 flushed
    between steps); returns the total device time in ms"""
    import torch
    with torch.cuda.stream(stream):
        for _ in range(max(warmup, 3)):
            batch.run()
        stream.synchronize()
        e0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        e1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        for s in range(steps):
            flush.fill_(float(s))
            e0[s].record(stream)
            batch.run()
            e1[s].record(stream)
        torch.cuda.synchronize()
    return sum(e0[s].elapsed_time(e1[s]) for s in range(steps))


# kernels of one batched step, whatever the number of segments (up to 2,048): closed forms with the
# counter reset, one cooperative level kernel per pair class, then beside each other the fix-up
# (collect, FP64 pass, spread, finish) and the potential stages (tier 1 with the self pairs, tier 2,
# tier 2b, the adaptive potential: seed, 12 depths, final sums; the adjacent pairs' P)
BATCH_LAUNCHES = 1 + 3 + 4 + (1 + 1 + 1 + (1 + 12 + 1) + 1)


def uneven_batch_section(args):
    """Many-mesh workload (C3): 48 seeded closed meshes of uneven size (500-60,000 triangles,
    log-uniform) and scale (5e-4 .. 1e2): ellipsoids, tori, jittered spheres; all four pair classes
    (near < 3h, lists built on the GPU, ordered as the reference's (i, j) rows followed by the
    reversed rows); relative 1e-6, mixed precision.  The batched form (every segment in one graph
    replay) against the same meshes run class by class through their own evaluators, all on one
    stream; CUDA events, 3 steps after 3 warm-up steps."""
    import torch
    from integrator2_gb300 import api, meshes
    mset = meshes.uneven_mesh_set(2026, 48, 500, 60000)
    stream = torch.cuda.Stream()
    evs, segs_dev, total, seg_of = [], [], 0, []
    batch = None
    for V, C, kind, scale in mset:
        m = api.Mesh3D()
        m.setGeometry(V, C)
        m.prepareMeshDevice(NEAR)
        it = api.NumericalIntegrator3D(m, api.qf3D13)
        it.setErrorControl(api.RELATIVE_ERROR_CONTROL, args.tol, 5)
        it.setPrecision(api.PRECISION_MIXED)
        ev = api.EvaluatorJ3DK(m, it)
        ev.setStream(stream.cuda_stream)
        unordered = [m.getSimpleNeighbors()[:, :2], m.getAttachedNeighbors()[:, :2], m.getNotNeighbors()[:, :2]]
        lists = [np.ascontiguousarray(np.concatenate([u, u[:, ::-1]])) for u in unordered]
        lists.append(np.ascontiguousarray(m.getSelfPairs()[:, :2]))
        dev = [(torch.from_numpy(l).to("cuda"), torch.empty(len(l), 3, dtype=torch.float64, device="cuda"),
                torch.empty(len(l), dtype=torch.float64, device="cuda")) for l in lists]
        if batch is None:
            batch = api.BatchEvaluator(it)
            batch.setStream(stream.cuda_stream)
        segs = [batch.add(m, c, l) for c, l in zip(CLASSES, lists)]
        evs.append((m, it, ev, dev))
        seg_of.append((V, C, scale, lists, segs))
        total += sum(len(l) for l in lists)

    def per_class_step():
        for m, it, ev, dev in evs:
            for c, (p, J, P) in zip(CLASSES, dev):
                if len(p):
                    ev.runClassDevice(c, p.data_ptr(), len(p), 0, J.data_ptr(), P.data_ptr())

    def timed(fn):
        with torch.cuda.stream(stream):
            for _ in range(3):
                fn()
            stream.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(3):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 3

    torch.cuda.synchronize()  # the lists were copied on torch's default stream; the runs use `stream`
    ms_per_class = timed(per_class_step)
    shape = batch.autotune()
    ms_batch = timed(batch.run)
    # accuracy of the batched results: 50 seeded pairs per class of six meshes (two of each
    # kind) against the oracle's high-order answer, on the geometry rescaled by a power of two
    # to unit size (J scales as s^2, P as s^3 exactly; the oracle's absolute thresholds then apply)
    rng = np.random.default_rng(13)
    acc = {}
    for mi in range(6):
        V, C, scale, lists, segs = seg_of[mi]
        s2 = 2.0 ** -round(np.log2(np.abs(V).max()))
        for c, l, sg in zip(CLASSES, lists, segs):
            if not len(l):
                continue
            idx = np.sort(rng.choice(len(l), min(50, len(l)), replace=False))
            a = class_accuracy(V * s2, C, c, l[idx], batch.getResults(sg)[idx] * s2 ** 2, batch.getPotentials(sg)[idx] * s2 ** 3)
            key = CLASS_NAMES[c]
            prev = acc.get(key)
            if prev is None:
                acc[key] = a
            else:
                for k2 in a:
                    if k2 != "sample" and k2 in prev:
                        prev[k2] = max(prev[k2], a[k2])
                prev["sample"] += a["sample"]
    sizes = [len(c) for _, c, _, _ in mset]
    return {"workload": "C3: 48 meshes (ellipsoids, tori, jittered geodesic spheres), 500-60000 triangles, scales 5e-4..1e2, near < 3h, relative 1e-6",
            "triangles": int(sum(sizes)), "triangles_per_mesh": [int(min(sizes)), int(max(sizes))], "pairs": int(total),
            "accuracy": {"vs": "oracle high-order answer (fixed level 4, adaptive potential 1e-10), 50 pairs per class of 6 meshes, "
                               "largest of the per-mesh figures", **acc},
            "batched": {"value": total / (ms_batch * 1e-3), "ms_per_step": ms_batch, "cuda_graph": batch.usesGraph(),
                        "shape": [int(x) for x in shape], "launches": f"{BATCH_LAUNCHES} for all {4 * len(mset)} segments"},
            "per_class": {"value": total / (ms_per_class * 1e-3), "ms_per_step": ms_per_class, "launches": "4 class chains x 48 meshes"}}


def local_fd(V, C, lists, c, w, k, h, loss, groups=None, **settings):
    """central difference of the loss with respect to coordinate k over the pairs that touch its
    vertex's cells (no other pair depends on that coordinate, so this equals the difference of the
    whole loss); groups: per class, the refinement level each pair is held at (a frozen
    refinement), None to run the settings as given"""
    import torch
    cells = np.where((np.asarray(C) == k // 3).any(axis=1))[0]
    sel = [np.isin(l[:, 0], cells) | np.isin(l[:, 1], cells) for l in lists]
    runs = []
    if groups is None:
        runs.append(([l[m] for l, m in zip(lists, sel)], [ck[m] for ck, m in zip(c, sel)], settings))
    else:
        for L in sorted({int(x) for g, m in zip(groups, sel) for x in np.asarray(g)[m]}):
            ms = [m & (np.asarray(g) == L) for g, m in zip(groups, sel)]
            runs.append(([l[m] for l, m in zip(lists, ms)], [ck[m] for ck, m in zip(c, ms)], dict(settings, mode="fixed", level=max(L, 0))))
    vals = []
    for sgn in (1.0, -1.0):
        Vp = np.array(V, np.float64).reshape(-1)
        Vp[k] += sgn * h
        Vq = torch.tensor(Vp.reshape(-1, 3), dtype=torch.float64, device="cuda")
        with torch.no_grad():
            vals.append(sum(float(loss(Vq, sub, cs, **kw)) for sub, cs, kw in runs))
    return (vals[0] - vals[1]) / (2 * h)


def adjoint_section(args):
    """C4 workload: 5,120-triangle sphere displaced radially by spherical harmonics of degree <= 6
    (coefficients ~ N(0, 0.05^2), seed 4), all four pair classes (near < 3h).  Times forward +
    backward of L = sum_p c_p (P_p + w . J_p) through the torch front-end (FP64 and FP32 adjoint)
    and checks both gradients against central differences (h = 1e-6) of the FP64 forward on
    --fd-coords seeded coordinates (each difference over the pairs that touch the coordinate's
    vertex, which equals the difference of the whole loss)."""
    import torch
    from integrator2_gb300 import api, meshes, pairs
    from integrator2_gb300.autograd import pair_integrals
    V, C = meshes.sh_displaced_icosphere(4, 6, 0.05, 4)
    pl = pairs.build_pairs(V, C, NEAR)
    lists = [pl.vertex, pl.edge, pl.far, pl.self_]
    rng = np.random.default_rng(11)
    c = [rng.standard_normal(len(l)) for l in lists]
    w = rng.standard_normal(3)
    wt = torch.as_tensor(w, device="cuda")
    settings = dict(mode="fixed", level=1, hard_tol=0.0)

    def loss(Vt, lst, cs, **kw):
        outs = pair_integrals(Vt, C, lst, **kw)
        return sum((torch.as_tensor(ck, device="cuda") * (P + J @ wt)).sum() for (J, P), ck in zip(outs, cs))

    out = {"workload": "C4: sphere s4 (5120 triangles) with SH displacement l<=6, 4 classes, fixed level 1",
           "pairs": int(sum(len(l) for l in lists))}
    grads = {}
    for name, prec in (("fp64", api.PRECISION_FP64), ("fp32", api.PRECISION_MIXED)):
        kw = dict(settings, precision=prec)
        times = []
        for rep in range(3):
            Vt = torch.tensor(V, dtype=torch.float64, device="cuda", requires_grad=True)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            L = loss(Vt, lists, c, **kw)
            t1 = time.perf_counter()
            L.backward()
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            times.append((t1 - t0, t2 - t1))
        fwd, bwd = np.median([t[0] for t in times]), np.median([t[1] for t in times])
        out[name] = {"forward_ms": 1e3 * fwd, "backward_ms": 1e3 * bwd}
        grads[name] = Vt.grad.detach().cpu().numpy().reshape(-1)
    h = 1e-6
    coords = rng.choice(V.size, max(1, args.fd_coords), replace=False)
    fd = np.array([local_fd(V, C, lists, c, w, int(k), h, loss, **settings) for k in coords])
    for name, g in grads.items():
        out[name]["fd_max_abs_err_over_max_grad"] = float(np.max(np.abs(fd - g[coords])) / np.abs(g).max())
    out["fd_check"] = {"coordinates": int(len(coords)), "h": h, "of": "FP64 forward",
                       "max_abs_err_over_max_grad": {n: out[n]["fd_max_abs_err_over_max_grad"] for n in grads}}
    out["fp32_vs_fp64_max_rel"] = float(np.abs(grads["fp32"] - grads["fp64"]).max() / np.abs(grads["fp64"]).max())
    return out


# DRAM bytes (read + write) of one run of the disjoint class's FP32 level chain (k_level_mixed<2>,
# levels 0..5 in five launches: levels 0 and 1 share one) on this workload, measured with ncu
# (dram__bytes_read.sum + dram__bytes_write.sum summed over the launches); the chain is
# compute-bound, this is mostly per-pair state
FAR_CHAIN_DRAM_BYTES = (21755136 + 32178944) + (46207744 + 6066688) + 1542144 + 120064 + 76288

# The algorithmic work of one far-field point, frozen from the reference's formula (thetaPsi,
# evaluatorJ3DK.cu:266-313; the hand count the roofline is defined on): about 150 flops, 3 sqrt,
# 12 divisions, 3 logs and 1 atan2; the transcendentals and divisions are weighted by their
# measured cost in the form's precision.  flops, sqrt, divide, log, atan2:
FROZEN_FAR = (150, 3, 12, 3, 1)
# the operations the kernels execute for the same point (the formulations avoid most divisions):
# FP32 far_field_integrand_f with the point's offsets (o_A interpolated, 15 flops; o_B and o_C from
# double-float edges, 12 flops), its divisions by |e| as multiplications, 3 quotients
POINT_OPS_F32 = {"far": (188, 3, 3, 3, 1)}


def point_flops_f32(cal, ops=None):
    a, sq, dv, lg, at = ops or POINT_OPS_F32["far"]
    return a + 2.0 * (sq * cal[8] + dv * cal[9] + lg * cal[10] + at * cal[11])


def point_flops_frozen(w):
    a, sq, dv, lg, at = FROZEN_FAR
    return a + sq * w["sqrt"] + dv * w["div"] + lg * w["log"] + at * w["atan2"]


def gpu_arm(args):
    import torch
    from integrator2_gb300 import api
    from integrator2_gb300._lib import lib

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    V, C, lists = workload()
    total = sum(len(v) for v in lists.values())

    cal = np.zeros(13)
    lib().i2_calibrate_pipes(cal.ctypes.data_as(ctypes.c_void_p))
    w = flop_weights(cal)

    m = api.Mesh3D()
    m.setGeometry(V, C)
    m.prepareMesh(NEAR)
    stream = torch.cuda.Stream()
    d_pairs = {c: torch.from_numpy(lists[c]).to("cuda") for c in CLASSES}
    d_J = {c: torch.empty(len(lists[c]), 3, dtype=torch.float64, device="cuda") for c in CLASSES}
    d_P = {c: torch.empty(len(lists[c]), dtype=torch.float64, device="cuda") for c in CLASSES}
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # inputs made on torch's default stream, evaluators run on `stream`

    forms = {}
    wanted = [f.strip() for f in args.forms.split(",") if f.strip()]
    for name, prec in (("fp64", api.PRECISION_FP64), ("mixed", api.PRECISION_MIXED)):
        if name not in wanted and not (name == "mixed" and "batch" in wanted):
            continue
        it = api.NumericalIntegrator3D(m, api.qf3D13)
        it.setErrorControl(api.RELATIVE_ERROR_CONTROL, args.tol, 5)
        it.setPrecision(prec)
        ev = api.EvaluatorJ3DK(m, it)
        ev.setStream(stream.cuda_stream)
        if world > 1:
            torch.distributed.barrier()
        with ClockSampler() as clk:
            ms, cls_ms = run_form(ev, lists, d_pairs, d_J, d_P, stream, flush, args.steps, args.warmup)
        if world > 1:
            t = torch.tensor([ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        J = {c: d_J[c].cpu().numpy() for c in CLASSES}
        P = {c: d_P[c].cpu().numpy() for c in CLASSES}
        levels = {}
        for c in CLASSES:
            ev.runClass(c, lists[c])  # host entry point: same results, records the kept level per pair
            levels[c] = ev.getLevels(c)
            if not np.array_equal(ev.getResults(c), J[c]):
                raise RuntimeError(f"{name}: host and device entry points disagree on class {c}")
        forms[name] = dict(ev=ev, it=it, ms=ms, cls_ms=cls_ms, J=J, P=P, levels=levels, clocks=clk.summary(),
                           value=total * world * args.steps / (ms * 1e-3))

    if "batch" in wanted:
        # batched form: the four classes as segments of one batch, one persistent cooperative
        # kernel for every refinement level, the whole step replayed as a CUDA graph
        it = forms["mixed"]["it"]
        batch = api.BatchEvaluator(it)
        batch.setStream(stream.cuda_stream)
        segs = {c: batch.add(m, c, lists[c]) for c in CLASSES}
        shape = batch.autotune()
        if world > 1:
            torch.distributed.barrier()
        with ClockSampler() as clk:
            ms = run_batch(batch, flush, stream, args.steps, args.warmup)
        if world > 1:
            t = torch.tensor([ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        J = {c: batch.getResults(segs[c]) for c in CLASSES}
        P = {c: batch.getPotentials(segs[c]) for c in CLASSES}
        levels = {c: batch.getLevels(segs[c]) for c in CLASSES}
        forms["batch"] = dict(ms=ms, J=J, P=P, levels=levels, clocks=clk.summary(), shape=shape, graph=batch.usesGraph(),
                              value=total * world * args.steps / (ms * 1e-3), cls_ms=forms["mixed"]["cls_ms"])

    head = forms["batch"] if "batch" in forms else forms[wanted[0]]
    per_class = forms["mixed"] if "mixed" in forms else forms[wanted[0]]
    ev = per_class["ev"]
    # e2e: host lists (pinned) -> H2D, compute, D2H of J and P inside the timed region
    h_pairs = {c: torch.from_numpy(lists[c]).pin_memory() for c in CLASSES}
    h_J = {c: torch.empty(len(lists[c]), 3, dtype=torch.float64).pin_memory() for c in CLASSES}
    h_P = {c: torch.empty(len(lists[c]), dtype=torch.float64).pin_memory() for c in CLASSES}
    h2d = sum(h_pairs[c].numel() * 4 for c in CLASSES)
    d2h = sum(h_J[c].numel() * 8 + h_P[c].numel() * 8 for c in CLASSES)
    e2e_ms = []
    # the copies overlap the compute: every class's lists go up on one copy stream, each class
    # starts when its list has arrived, and its J and P come down on another copy stream while the
    # next class computes; the disjoint class (the largest results) runs first, so its download
    # hides behind the adjacent classes
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    order = [2, 0, 1, 3]
    for s in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(s))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        arrived = {}
        with torch.cuda.stream(up):
            for c in order:
                d_pairs[c].copy_(h_pairs[c], non_blocking=True)
                arrived[c] = torch.cuda.Event()
                arrived[c].record(up)
        for c in order:
            stream.wait_event(arrived[c])
            ev.runClassDevice(c, d_pairs[c].data_ptr(), len(lists[c]), 0, d_J[c].data_ptr(), d_P[c].data_ptr())
            done = torch.cuda.Event()
            done.record(stream)
            down.wait_event(done)
            with torch.cuda.stream(down):
                h_J[c].copy_(d_J[c], non_blocking=True)
                h_P[c].copy_(d_P[c], non_blocking=True)
        down.synchronize()
        stream.synchronize()
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_value = total * world / (np.median(e2e_ms) * 1e-3)
    if rank != 0:
        return

    def far_roofline(form, per_point, per_point_exec, peak, unit_note):
        lev = form["levels"][2]
        evals = int(sum(np.sum(lev >= L) * 4 ** L for L in range(6)))
        seconds = form["cls_ms"][2] * 1e-3
        achieved = evals * 13 * per_point / seconds / 1e12
        executed = evals * 13 * per_point_exec / seconds / 1e12
        return {"achieved": achieved, "peak": peak, "frac": achieved / peak, "flops_per_point": per_point,
                "point_evaluations": evals * 13, "note": unit_note,
                "executed_ops": {"flops_per_point": per_point_exec, "achieved": executed, "frac": executed / peak,
                                 "note": "the operations the kernel performs per point (fewer divisions than the frozen formula)"}}

    roof = {}
    frozen_note = "frozen per-point work of the reference's far-field formula: 150 flops, 3 sqrt, 12 div, 3 log, 1 atan2"
    if "mixed" in forms:
        w32 = {"sqrt": 2.0 * cal[8], "div": 2.0 * cal[9], "log": 2.0 * cal[10], "atan2": 2.0 * cal[11]}
        roof["mixed"] = far_roofline(forms["mixed"], point_flops_frozen(w32), point_flops_f32(cal), float(cal[1]),
                                     "FP32 FMA peak measured live (i2_calibrate_pipes); " + frozen_note)
    if "fp64" in forms:
        roof["fp64"] = far_roofline(forms["fp64"], point_flops_frozen(w), point_flops("far", w), float(cal[0]),
                                    "FP64 FMA peak measured live; " + frozen_note)
    acc = {name: accuracy(V, C, lists, f["J"], f["P"], f["levels"]) for name, f in forms.items()}
    population = {name: full_population(lists, f, forms["fp64"]) for name, f in forms.items()
                  if name != "fp64" and "fp64" in forms}
    n_cpu, dt_cpu, thr = cpu_run(V, C, lists, args.cpu_fraction, args.tol)
    # kernels per step: adjacent classes run singular + tiers 2 and 2b + adaptive potential (seed,
    # 12 depths, final); per-class chains add levels 0..5 + finalize per class, self pairs 1; the
    # mixed chains add tier 1 as its own kernel and the needle fix-up (collect, FP64 pass, spread,
    # finish) per non-self class.  The batched form: BATCH_LAUNCHES.
    pot_chain = 4 + 12
    launches = {"fp64": 2 * (1 + pot_chain + 7) + 7 + 1, "mixed": 2 * (2 + pot_chain + 7) + 7 + 1 + 3 * 4, "batch": BATCH_LAUNCHES}
    names4 = ("vertex", "edge", "near", "self")
    form_desc = {"batch": "mixed precision, batched: 4 class segments, one persistent cooperative level kernel, CUDA graph replay",
                 "mixed": "mixed precision, per-class kernel chains", "fp64": "plain FP64, per-class kernel chains"}
    hname = "batch" if "batch" in forms else wanted[0]
    line = {
        "metric": METRIC, "value": head["value"], "unit": "pair-integrals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if hname == "fp64" else "f32 bulk / f64 singular, estimator and hard pairs",
        "data": "synthetic",
        "config": workload_config(total, args.tol),
        "form": form_desc[hname], "l2": "flushed (512 MiB write) between steps", "parallelism": f"replicas x{world}",
        "e2e": {"value": e2e_value, "unit": "pair-integrals/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "path": "EvaluatorJ3DK device entry point per class (mixed precision), pinned host lists in, J and P out; "
                        "uploads and downloads on their own streams, overlapping the classes' compute"},
        "forms": {n: {"value": f["value"], "ms_per_step": f["ms"] / args.steps,
                      "class_ms": dict(zip(names4, map(float, f["cls_ms"]))) if n != "batch" else None,
                      "accuracy": acc[n], "gpu_launches_per_step": launches[n]} for n, f in forms.items()},
        "accuracy": acc[hname],
        "accuracy_all_pairs_vs_fp64": population.get(hname),
        "accuracy_statement": accuracy_statement(population.get(hname), acc[hname]),
        "levels": {n: np.bincount(head["levels"][c][head["levels"][c] >= 0], minlength=6).tolist() for n, c in
                   zip(("vertex", "edge", "near"), (0, 1, 2))},
        "calibration": {"fp64_tflops": float(cal[0]), "fp32_tflops": float(cal[1]),
                        "fp64_fma_units": dict(zip(("sqrt", "div", "log", "atan2", "sincos", "acos"), map(float, cal[2:8]))),
                        "fp32_fma_units": dict(zip(("sqrtf", "div", "log1pf", "atan2f", "logf"), map(float, cal[8:13])))},
        "cpu_baseline": {"value": n_cpu / dt_cpu, "unit": "pair-integrals/s", "cores": thr, "kind": "port",
                         "sample": (f"every pair ({n_cpu})" if args.cpu_fraction >= 1 else
                                    f"{args.cpu_fraction:.3f} of every class ({n_cpu} pairs)") + ", oracle C restatement, OpenMP, same rules"},
        "clocks": head["clocks"],
        "gpu_launches": launches[hname] * args.steps,
    }
    if "fp64" in forms:
        line["speedup_over_plain_fp64"] = head["value"] / forms["fp64"]["value"]
    sections = {x.strip() for x in args.sections.split(",") if x.strip()}
    if "uneven" in sections:
        line["uneven_batch"] = uneven_batch_section(args)
    if "c5" in sections:
        line["c5"] = c5_section(args)
    if "level0" in sections:
        line["level0_j_only"] = {"fp64": level0_j_only(stream, api.PRECISION_FP64), "mixed": level0_j_only(stream, api.PRECISION_MIXED),
                                 "note": "the reference's own workload (J only, fixed level 0, qf3D13, its three classes); "
                                         "--impl reference times the reference's CUDA build on it (reference_cuda)"}
    if "adjoint" in sections:
        line["adjoint"] = adjoint_section(args)
    if "examples" in sections:
        line["example_surfaces_mixed_vs_fp64"] = example_surfaces_section()
    if "batch" in forms:
        line["batch"] = {"shape": {"threads": forms["batch"]["shape"][0], "blocks_per_sm": forms["batch"]["shape"][1],
                                   "lanes_per_pair": forms["batch"]["shape"][2],
                                   "registers": {name: {0: "unconstrained", 1: "capped at 128", 2: "capped at 85"}[
                                       (int(forms["batch"]["shape"][3]) // place) % 3]
                                                 for name, place in (("vertex", 1), ("edge", 3), ("near", 9))}},
                         "cuda_graph": forms["batch"]["graph"]}
    rk = "mixed" if "mixed" in roof else ("fp64" if "fp64" in roof else None)
    if rk:
        line["roofline"] = {"bound": "fp32" if rk == "mixed" else "fp64",
                            "kernel": ("k_level_mixed" if rk == "mixed" else "k_level") + "<far> chain (levels 0..5), per-class form; "
                                      "timed over the whole disjoint class (chain, finalisation, needle fix-up)",
                            "unit": "TFLOP/s", "traffic": FAR_CHAIN_DRAM_BYTES if rk == "mixed" else None,
                            "traffic_unit": "bytes per chain run (ncu)", **roof[rk]}
    if "fp64" in roof and rk != "fp64":
        line["roofline_fp64"] = {"bound": "fp64", "unit": "TFLOP/s", **roof["fp64"]}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--cpu-fraction", type=float, default=1.0,
                    help="cpu_baseline leg of the GPU arm: share of every class (1 = every pair, about 2.5 s on 16 cores)")
    ap.add_argument("--fd-coords", type=int, default=200, help="adjoint section: coordinates checked by finite differences")
    ap.add_argument("--c5-backward-fraction", type=float, default=0.05,
                    help="c5 section: share of every class's pairs the timed backward pass covers (1 = all 194 M pairs, minutes)")
    ap.add_argument("--forms", default="fp64,mixed,batch",
                    help="forms to run: fp64, mixed (per-class chains), batch (headline when present)")
    ap.add_argument("--sections", default="uneven,c5,adjoint,level0,examples",
                    help="side sections after the C2 line: uneven (48 meshes, batched vs per class), c5 (2 M triangles), "
                         "adjoint (C4), level0 (plain FP64, J only, fixed level 0 on C1/C2: the reference's own "
                         "workload; --impl reference times the reference's CUDA build on it), examples (mixed vs FP64 "
                         "on the reference's example surfaces); empty for the C2 line alone")
    args = ap.parse_args()
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
