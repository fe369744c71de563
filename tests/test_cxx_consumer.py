"""The C++ drop-in layer: a program in the reference's call pattern compiles against
include/integrator2_gb300.hpp, links libi2gb300.so and runs its host-side part."""
import os
import subprocess

import numpy as np
import pytest

from tests._util import ROOT, ensure_built


def _build(tmp_path):
    so = ensure_built()
    exe = tmp_path / "consumer"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cxx", "consumer.cpp"),
                        "-o", str(exe), "-L", os.path.dirname(so), "-li2gb300", "-Wl,-rpath," + os.path.dirname(so)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_consumer_host_part(tmp_path):
    from integrator2_gb300 import meshes, pairs
    exe = _build(tmp_path)
    V, C = meshes.icosphere(1)
    dat = tmp_path / "m.dat"
    meshes.write_dat(str(dat), V, C)
    r = subprocess.run([str(exe), str(dat), "host"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    pl = pairs.build_pairs(V, C, near_factor=None)
    line = [l for l in r.stdout.splitlines() if l.startswith("pairs")][0].split()[1:]
    assert list(map(int, line)) == [len(pl.vertex) // 2, len(pl.edge) // 2, len(pl.far) // 2, len(C)]


@pytest.mark.gpu
def test_consumer_runs_all_pairs(tmp_path):
    from integrator2_gb300 import meshes
    exe = _build(tmp_path)
    V, C = meshes.icosphere(1)
    dat = tmp_path / "m.dat"
    meshes.write_dat(str(dat), V, C)
    r = subprocess.run([str(exe), str(dat), "run"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "AttachedNeighbors.csv").exists()
