"""Generates the golden vectors in tests/golden/ from the REFERENCE's own routines.

Run here (where the reference checkout exists), not on the GPU machine:

    python tests/golden/gen_golden.py            # reference at /root/reference
    I2_REFERENCE=/path/to/integrator2 python tests/golden/gen_golden.py
    python tests/golden/gen_golden.py --only-all # only the all-disjoint fixture (ico1_all.npz)
    python tests/golden/gen_golden.py --only-examples  # only the example-mesh fixtures (cubehole.npz, examples.npz)

It builds oracle/_ref/libi2ref.so (oracle/ref_build.sh: the reference's src/ compiled for the
host through oracle/ref_shim.h, plus oracle/ref_driver.cu, which mirrors the reference's kernel
bodies and its host refinement loop) and records, per mesh and pair class, the reference's
results in three modes: fixed refinement level 0, fixed level 1 and automatic error control.
Inputs (vertices, cells, pair lists) are stored beside the outputs so the tests need nothing
but the .npz files.

The two-triangle meshes are the reference's own examples/Case-*.dat stress fixtures (read with
the reference's .dat semantics).  In the coplanar common-edge branch the reference leaves
q_theta unset (evaluatorJ3DK.cu:474-481); tasks that take that branch are flagged in
``uninit_theta`` and their Theta is not compared.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from integrator2_gb300 import meshes as M  # noqa: E402
from integrator2_gb300 import pairs as P  # noqa: E402
from oracle import oracle as O  # noqa: E402

REF = os.environ.get("I2_REFERENCE", "/root/reference")
CLASSES = (O.VERTEX, O.EDGE, O.FAR)


def coplanar_edge_branch(V, C, pairs):
    """Tasks whose closed form takes the coplanar branch: |xi| < 1e-6 and a matching angle."""
    n, _, _ = O.cell_geometry(V, C)
    flags = np.zeros(len(pairs), bool)
    for k, (i, j) in enumerate(pairs):
        xi = abs(np.arctan2(np.linalg.norm(np.cross(n[i], n[j])), np.dot(n[i], n[j])))
        flags[k] = xi < 1e-6
    return flags


def run_mesh(name, V, C, pl: P.PairLists, far_sample=None, seed=0, modes=(0, 1, -1), sample=None):
    """sample: at most this many pairs of every class (seeded); far_sample: of the disjoint class"""
    out = {"V": V, "C": C.astype(np.int32)}
    rng = np.random.default_rng(seed)
    for cls in CLASSES:
        pairs = pl.by_class(cls)
        cap = far_sample if cls == O.FAR and far_sample is not None else sample
        if cap is not None and len(pairs) > cap:
            pairs = pairs[np.sort(rng.choice(len(pairs), cap, replace=False))]
        if len(pairs) == 0:
            continue
        out[f"pairs_{cls}"] = pairs.astype(np.int32)
        for lev in modes:
            raw, J, it = O.ref_integrate(cls, pairs, V, C, level=lev)
            tag = {0: "L0", 1: "L1", -1: "adaptive"}[lev]
            out[f"J_{cls}_{tag}"] = J
            if lev == 0:
                out[f"raw_{cls}_{tag}"] = raw
            if lev == -1:
                out[f"iters_{cls}_{tag}"] = it.astype(np.int8)
        if cls == O.EDGE:
            out[f"uninit_theta_{cls}"] = coplanar_edge_branch(V, C, pairs)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: " + ", ".join(f"{k}={v.shape}" for k, v in out.items() if k.startswith("pairs")))


def all_disjoint(name, V, C):
    """every disjoint pair, the rows runAllPairs integrates (evaluator3d.cu:120-204: the full
    not-neighbours list plus its reversed rows, kAddReversedPairs at :22-31), as ordered pairs
    sorted i-major (the reference's list order comes from atomics, so tests match rows by
    (i, j)); the reference's J at fixed levels 0 and 1"""
    pl = P.build_pairs(V, C, near_factor=None)
    rows = pl.far.astype(np.int32)
    out = {"V": V, "C": C.astype(np.int32), "pairs": rows}
    for lev in (0, 1):
        out[f"J_L{lev}"] = O.ref_integrate(O.FAR, rows, V, C, level=lev)[1]
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: {len(rows)} ordered disjoint pairs")


def point_samples(n=400, seed=11):
    """theta/psi of the reference at seeded points around a seeded triangle, including points
    close to the triangle's plane, edges and vertices."""
    rng = np.random.default_rng(seed)
    R = O.ref_lib()
    rows = []
    for _ in range(n):
        A, B, C = rng.normal(size=(3, 3))
        kind = rng.integers(4)
        if kind == 0:
            x = rng.normal(size=3) * 2.0
        else:
            bary = rng.dirichlet([1, 1, 1])
            x = bary @ np.stack([A, B, C])
            nrm = np.cross(B - A, C - A)
            nrm /= np.linalg.norm(nrm)
            x = x + nrm * (10.0 ** -rng.uniform(1, 6)) * rng.choice([-1, 1]) + \
                (rng.normal(size=3) * 0.3 if kind == 3 else 0)
        out = np.zeros(4)
        R.refd_theta_psi(O._p(x), O._p(A), O._p(B), O._p(C), O._p(out))
        rows.append(np.concatenate([x, A, B, C, out]))
    return np.asarray(rows)


# the reference's example surfaces (README.md "Noticeable examples") at the scales it gives
EXAMPLES = (("G1", "G1.dat", 1.0), ("Krylo01", "Krylo01.dat", 1.0), ("Girja", "Girja.dat", 1.0),
            ("ellipsoid2000", "ellipsoid2000", 1.0), ("Fish", "Fish.dat", 100.0), ("s5m", "s5m.dat", 0.0005))


def example_meshes():
    """the reference's cubehole.dat example (a unit cube with a square hole: coplanar faces and
    90-degree folds), its near-field classes at fixed levels 0 and 1; and its example surfaces
    at their scales, 800 seeded pairs of every class (examples.npz, keys "<mesh>|<field>")"""
    V, C = M.read_dat(os.path.join(REF, "examples", "cubehole.dat"))
    run_mesh("cubehole", V, C, P.build_pairs(V, C), far_sample=2500, seed=4, modes=(0, 1))
    flat = {}
    for k, (nm, fname, scale) in enumerate(EXAMPLES):
        V, C = M.read_dat(os.path.join(REF, "examples", fname), scale)
        run_mesh("_example", V, C, P.build_pairs(V, C), seed=10 + k, modes=(0, 1), sample=800)
        path = os.path.join(HERE, "_example.npz")
        with np.load(path) as d:
            for key in d.files:
                flat[f"{nm}|{key}"] = d[key]
        os.remove(path)
    np.savez_compressed(os.path.join(HERE, "examples.npz"), **flat)
    print(f"examples: {len(EXAMPLES)} surfaces")


def main():
    subprocess.run([os.path.join(ROOT, "oracle", "ref_build.sh")], check=True,
                   env=dict(os.environ, I2_REFERENCE=REF))
    if O.ref_lib() is None:
        raise SystemExit("reference host library not built")
    if "--only-examples" in sys.argv:
        example_meshes()
        return
    # full not-neighbours semantics (prepareMesh without a near-field cutoff + runAllPairs) on a
    # jittered 80-cell sphere
    V, C = M.jittered_icosphere(1, 0.15, 5)
    all_disjoint("ico1_all", V, C)
    if "--only-all" in sys.argv:
        return
    # C1 workload: icosphere subdivided twice, radius 1
    V, C = M.icosphere(2)
    run_mesh("ico2", V, C, P.build_pairs(V, C), far_sample=2500, seed=1, modes=(0, 1))
    # jittered icosphere (seed 7, sigma = 0.15 h)
    V, C = M.jittered_icosphere(2, 0.15, 7)
    run_mesh("ico2_jitter", V, C, P.build_pairs(V, C), far_sample=2500, seed=2)
    # scaled copy: the reference's absolute tolerances are meant for meshes of size 1..100
    V, C = M.jittered_icosphere(1, 0.15, 3, radius=20.0)
    run_mesh("ico1_r20", V, C, P.build_pairs(V, C), far_sample=1200, seed=3)
    # two-triangle stress fixtures of the reference
    case = {}
    for path in sorted(glob.glob(os.path.join(REF, "examples", "Case*.dat")) +
                       [os.path.join(REF, "examples", f) for f in ("Test.dat", "G1new.dat", "G1contactR.dat", "genCase.dat")]):
        if not os.path.exists(path):
            continue
        V, C = M.read_dat(path)
        if len(C) != 2:
            continue
        pl = P.build_pairs(V, C, near_factor=None)
        nm = os.path.basename(path)[:-4]
        for cls in CLASSES:
            pairs = pl.by_class(cls)
            if len(pairs) == 0:
                continue
            r0 = O.ref_integrate(cls, pairs, V, C, level=0)
            r1 = O.ref_integrate(cls, pairs, V, C, level=1)
            ra = O.ref_integrate(cls, pairs, V, C, level=-1)
            case[nm] = dict(V=V, C=C, cls=cls, pairs=pairs, raw_L0=r0[0], J_L0=r0[1], J_L1=r1[1], J_adaptive=ra[1],
                            iters=ra[2], uninit=coplanar_edge_branch(V, C, pairs) if cls == O.EDGE else np.zeros(len(pairs), bool))
    flat = {}
    for nm, d in case.items():
        for k, v in d.items():
            flat[f"{nm}|{k}"] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "cases.npz"), **flat)
    print(f"cases: {len(case)} two-triangle fixtures")
    np.savez_compressed(os.path.join(HERE, "theta_psi_points.npz"), rows=point_samples())
    print("theta_psi_points: 400 samples")
    example_meshes()


if __name__ == "__main__":
    main()
