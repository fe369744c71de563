"""The C++ source drop-in (include/integrator2/: the reference's header names and classes over the
C-ABI).  The reference's own test program compiles unchanged against it (where the reference
checkout exists), and a program in the reference's call pattern with a harness subclass of
EvaluatorJ3DK builds with g++ and, on a GPU, gives the Python API's results."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests._util import ROOT, ensure_built, reference_checkout


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _build_consumer(tmp_path):
    so = ensure_built()
    exe = tmp_path / "consumer"
    cuda = _cuda_home()
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
                        os.path.join(ROOT, "tests", "cxx", "consumer.cpp"), "-o", str(exe), "-L", os.path.dirname(so), "-li2gb300",
                        "-Wl,-rpath," + os.path.dirname(so), "-L", os.path.join(cuda, "lib64"), "-lcudart"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_consumer_builds_with_the_dropin_headers(tmp_path):
    """host C++ (g++) against include/integrator2/ and libi2gb300.so"""
    assert _build_consumer(tmp_path).exists()


def test_reference_test_program_compiles_unchanged(tmp_path):
    """the reference's tests/integrator3D/main.cu, copied unmodified into a tree whose src/ is this
    library's header set (its includes are ../../src/Mesh3d.cuh and the others), compiles, links
    against libi2gb300.so and prints its usage"""
    ref = reference_checkout()
    if ref is None:
        pytest.skip("no reference checkout recorded by oracle/ref_build.sh")
    so = ensure_built()
    (tmp_path / "tests" / "integrator3D").mkdir(parents=True)
    os.symlink(os.path.join(ROOT, "include", "integrator2"), tmp_path / "src")
    os.symlink(os.path.join(ref, "thirdparty"), tmp_path / "thirdparty")
    main = tmp_path / "tests" / "integrator3D" / "main.cu"
    shutil.copyfile(os.path.join(ref, "tests", "integrator3D", "main.cu"), main)
    exe = tmp_path / "integrator2test3D"
    r = subprocess.run(["nvcc", "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", "-diag-suppress", "20091,20092",
                        str(main), "-o", str(exe), "-L", os.path.dirname(so), "-li2gb300", "-Xlinker", "-rpath=" + os.path.dirname(so)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([str(exe), "--help"], capture_output=True, text=True)
    assert out.returncode == 0 and "--meshfile" in out.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("level", [1, -1])
def test_consumer_matches_python_api(tmp_path, level):
    """the harness subclass's full-precision results (runAllPairs with the antisymmetry check, the
    rows of the reference's task lists) equal the Python API's runAllPairs results; the refined
    mesh export has the reference's vertex and cell counts"""
    from integrator2_gb300 import api, meshes
    exe = _build_consumer(tmp_path)
    V, C = meshes.jittered_icosphere(1, 0.15, 3)
    dat = tmp_path / "m.dat"
    meshes.write_dat(str(dat), V, C)
    r = subprocess.run([str(exe), str(dat), str(level), str(tmp_path / "out.txt")], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = np.loadtxt(tmp_path / "out.txt")
    m = api.Mesh3D()
    m.loadMeshFromFile(str(dat))
    m.prepareMesh(None)
    it = api.NumericalIntegrator3D(m, api.qf3D13)
    if level >= 0:
        it.setFixedRefinementLevel(level)
    ev = api.EvaluatorJ3DK(m, it)
    ev.runAllPairs(True)
    for cls in (0, 1, 2):
        got = rows[rows[:, 0] == cls]
        J = ev.getResults(cls)
        assert len(got) == len(J)
        lst = [m.getSimpleNeighbors, m.getAttachedNeighbors, m.getNotNeighbors][cls]()[:, :2]
        assert np.array_equal(got[:, 1:3].astype(int), np.concatenate([lst, lst[:, ::-1]]))
        assert np.array_equal(got[:, 3:6], J), cls
        assert np.allclose(got[:, 6], ev.getErrors(cls), rtol=1e-12, atol=1e-15), cls
    assert (tmp_path / "AttachedNeighbors.csv").exists()
    nv, nc = len(V), len(C)
    L = max(level, 0)
    assert f"refined {nv + nc * (4 ** L - 1)} {nc * 4 ** L}" in r.stdout
