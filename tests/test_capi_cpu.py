"""C-ABI checks that need no GPU: the library loads, exports every symbol of
include/integrator2_gb300.h, and its host-side logic (built-in rules, .dat reader, O(N) pair
builder) agrees with the reference's semantics."""
import ctypes
import os

import numpy as np
import pytest

from tests._util import declared_symbols, ensure_built


@pytest.fixture(scope="module")
def lib():
    ensure_built()
    from integrator2_gb300 import _lib
    return _lib.lib()


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 30
    from integrator2_gb300 import _lib
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"


def test_builtin_rules_match_reference_tables():
    from integrator2_gb300.api import QuadratureFormula3D
    from oracle.oracle import QF13
    q = QuadratureFormula3D.builtin(13)
    assert q.order == 7
    np.testing.assert_array_equal(q.coordinates, QF13[0])
    np.testing.assert_array_equal(q.weights, QF13[1])
    for n, order in ((1, 2), (3, 2), (4, 3), (6, 4), (7, 5), (9, 5), (12, 6)):
        r = QuadratureFormula3D.builtin(n)
        assert r.order == order and len(r.weights) == n
        assert abs(r.weights.sum() - 1.0) < 1e-12
    with pytest.raises(Exception):
        QuadratureFormula3D.builtin(5)


def test_status_codes_and_messages(lib):
    from integrator2_gb300 import api
    m = api.Mesh3D()
    assert not m.loadMeshFromFile("/nonexistent/file.dat")
    assert "cannot open" in api.lastError()
    with pytest.raises(Exception):
        m.setGeometry(np.zeros((3, 3)), np.array([[0, 1, 5]]))  # vertex 5 missing
    with pytest.raises(Exception):
        m.getSimpleNeighbors()  # not prepared


@pytest.mark.parametrize("near", [None, 3.0])
def test_pair_lists_match_python_builder(lib, near):
    from integrator2_gb300 import api, meshes, pairs
    V, C = meshes.jittered_icosphere(3, 0.15, 5)
    m = api.Mesh3D()
    m.setGeometry(V, C)
    m.prepareMesh(near)
    pl = pairs.build_pairs(V, C, near_factor=near)
    for cls, got in ((pairs.VERTEX, m.getSimpleNeighbors()), (pairs.EDGE, m.getAttachedNeighbors()),
                     (pairs.FAR, m.getNotNeighbors())):
        ref = pl.by_class(cls)
        ref = ref[ref[:, 0] < ref[:, 1]]
        assert np.array_equal(got[:, :2], ref), cls
        assert np.array_equal(got[:, 2], np.arange(len(got)))
    assert len(m.getSelfPairs()) == len(C)
    n, s, c = m.getCellNormals(), m.getCellMeasures(), m.getCellCenters()
    from oracle.oracle import cell_geometry
    on, os_, oc = cell_geometry(V, C)
    assert np.abs(n - on).max() < 1e-15 and np.abs(s - os_).max() < 1e-16 and np.abs(c - oc).max() < 1e-15


def test_dat_reader_semantics(lib, tmp_path):
    """The reference's loader keeps (header count - skipped elements) triangles; non-triangle
    elements (type != 203) consume four tokens (src/Mesh3d.cu:159-217)."""
    from integrator2_gb300 import api, meshes
    V, C = meshes.icosphere(0)
    p = tmp_path / "m.dat"
    meshes.write_dat(str(p), V, C)
    m = api.Mesh3D()
    assert m.loadMeshFromFile(str(p), 2.0)
    m.prepareMesh(None)
    assert m.sizes() == (12, 20)
    area = 0.5 * np.linalg.norm(np.cross(V[C[:, 1]] - V[C[:, 0]], V[C[:, 2]] - V[C[:, 0]]), axis=1)
    assert np.allclose(m.getCellMeasures(), 4.0 * area, rtol=1e-14)
    # a line element (type 102) in the middle and no trailing newline
    text = "4 3\n1 0 0 0\n2 1 0 0\n3 0 1 0\n4 0 0 1\n1 203 1 2 3\n2 102 1 2\n3 203 1 2 4"
    q = tmp_path / "q.dat"
    q.write_text(text)
    assert m.loadMeshFromFile(str(q))
    m.prepareMesh(None)
    assert m.sizes() == (4, 2)
    Vr, Cr = meshes.read_dat(str(q))
    assert len(Cr) == 2
    # trailing whitespace after a triangle: the extra loop turn re-reads type 203, count unchanged
    q.write_text(text + "\n")
    assert m.loadMeshFromFile(str(q))
    m.prepareMesh(None)
    assert m.sizes() == (4, 2)
    # degenerate cell is rejected at prepare
    m.setGeometry(np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0.0]]), np.array([[0, 1, 2]]))
    with pytest.raises(Exception):
        m.prepareMesh(None)


def test_integrator_argument_checks(lib):
    from integrator2_gb300 import api, meshes
    m = api.Mesh3D()
    V, C = meshes.icosphere(1)
    m.setGeometry(V, C)
    m.prepareMesh(3.0)
    it = api.NumericalIntegrator3D(m, api.qf3D13)
    assert it.getErrorControlType() == api.AUTOMATIC_ERROR_CONTROL
    it.setFixedRefinementLevel(1)
    assert it.getErrorControlType() == api.FIXED_REFINEMENT_LEVEL
    with pytest.raises(Exception):
        it.setFixedRefinementLevel(-1)
    with pytest.raises(Exception):
        it.setErrorControl(api.RELATIVE_ERROR_CONTROL, 0.0, 3)
    with pytest.raises(Exception):
        it.setPotentialRule(40, 8, 3, 16)
