"""The command-line driver (integrator2test3D, the reference's test-program options) built by
build(): argument handling on the CPU; a full run on a small mesh on the GPU, its CSV results
against the library's API and its mesh exports."""
import os
import subprocess

import numpy as np
import pytest

from tests._util import ROOT, ensure_built

EXE = os.path.join(ROOT, "integrator2_gb300", "integrator2test3D")


@pytest.fixture(scope="module")
def exe():
    ensure_built()
    from integrator2_gb300.build import build_cli
    return build_cli()


def test_cli_arguments(exe, tmp_path):
    r = subprocess.run([exe, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "USAGE: integrator2test3D" in r.stdout and "--checkresults" in r.stdout
    r = subprocess.run([exe, "--bogus"], capture_output=True, text=True)
    assert r.returncode != 0 and "Unknown option" in r.stderr
    r = subprocess.run([exe, "-s", "abc", "-f", "x.dat"], capture_output=True, text=True)
    assert r.returncode != 0 and "numeric" in r.stderr
    r = subprocess.run([exe, "-c"], capture_output=True, text=True)
    assert r.returncode != 0 and "No input file" in r.stdout
    r = subprocess.run([exe, "-f", str(tmp_path / "missing.dat")], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode != 0


@pytest.mark.gpu
def test_cli_run_matches_api(exe, tmp_path):
    from integrator2_gb300 import api, meshes
    V, C = meshes.jittered_icosphere(1, 0.1, 3)
    dat = tmp_path / "m.dat"
    meshes.write_dat(str(dat), V, C)
    r = subprocess.run([exe, "-f", str(dat), "-r", "1", "-c", "--exporttocsv", "--fullprecision", "--exporttoobj", "--exporttovtk"],
                       capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Using fixed refinement level equal to 1" in r.stdout
    assert "largest (i,j)/(j,i) difference" in r.stdout
    m = api.Mesh3D()
    m.setGeometry(V, C)
    m.prepareMesh(0.0)
    it = api.NumericalIntegrator3D(m, api.qf3D13)
    it.setFixedRefinementLevel(1)
    ev = api.EvaluatorJ3DK(m, it)
    ev.runAllPairs(True)
    for cls, name in ((0, "SimpleNeighbors"), (1, "AttachedNeighbors"), (2, "NotNeighbors")):
        rows = np.genfromtxt(tmp_path / f"{name}.csv", delimiter=";", skip_header=1)
        assert np.array_equal(rows[:, 2:5], ev.getResults(cls)), name
    obj = (tmp_path / "RefinedMesh.obj").read_text().splitlines()
    assert sum(l.startswith("f ") for l in obj) == 4 * len(C)
    assert sum(l.startswith("v ") for l in (tmp_path / "OriginalMesh.obj").read_text().splitlines()) == len(V)
    assert (tmp_path / "RefinedMesh.vtp").exists()
    # adaptive run: the VTK export carries per-cell refinement levels
    r = subprocess.run([exe, "-f", str(dat), "--exporttovtk"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "SimpleNeighborsRefinements" in (tmp_path / "OriginalMesh.vtp").read_text()
