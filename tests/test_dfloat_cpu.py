"""Accuracy of the double-float arithmetic the mixed form's potential stages compute in
(integrator2_gb300/csrc/i2_dfloat.cuh): the header compiled for the host by g++ runs seeded random
operands through +, -, *, /, sqrt, log, atan2, sin, cos, tan and acos and compares them with long
double.  Bars: a few u^2 (u = 2^-24) for the arithmetic and the square root, 2^-43 relative for
the transcendental functions (sin and cos away from their zeros, 2^-46 absolute everywhere);
atan2 keeps the C library's signed-zero and quadrant conventions.  Also checks the generated tables are current."""
import os
import subprocess

import pytest

from tests._util import ROOT

CSRC = os.path.join(ROOT, "integrator2_gb300", "csrc")
U2 = 2.0 ** -48


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    exe = tmp_path_factory.mktemp("df") / "dfloat_check"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", CSRC, os.path.join(ROOT, "tests", "cxx", "dfloat_check.cpp"),
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    return {ln.split()[0]: (int(ln.split()[1]), float(ln.split()[2])) for ln in out.splitlines()}


@pytest.mark.parametrize("op,bar", [("add", 3 * U2), ("sub", 3 * U2), ("mul", 5 * U2), ("div", 10 * U2), ("sqrt", 10 * U2),
                                    ("log", 2.0 ** -43), ("log_near_1", 2.0 ** -43), ("atan2", 2.0 ** -43),
                                    ("atan2_small", 2.0 ** -43), ("sin", 2.0 ** -43), ("cos", 2.0 ** -43), ("tan", 2.0 ** -43),
                                    ("acos", 2.0 ** -43), ("sin_small", 2.0 ** -43), ("sin_abs", 2.0 ** -46)])
def test_dfloat_accuracy(results, op, bar):
    n, err = results[op]
    assert n >= 100000 and err <= bar, (op, err, bar)


def test_atan2_signed_zeros(results):
    assert results["signed_zeros"][1] == 1


def test_tables_current(tmp_path):
    """gen_dftables.py reproduces the committed i2_dftables.h"""
    import importlib.util
    with open(os.path.join(CSRC, "i2_dftables.h")) as f:
        committed = f.read()
    spec = importlib.util.spec_from_file_location("gen_dftables_check", os.path.join(CSRC, "gen_dftables.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.HERE = str(tmp_path)
    mod.main()
    assert (tmp_path / "i2_dftables.h").read_text() == committed
