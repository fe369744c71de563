"""The GPU pair-list builder (i2_mesh_prepare_device) against the host builder
(i2_mesh_prepare): the same four lists in the same order, bit for bit, on closed and open meshes,
high-valence vertices, tiny scales, near-field and all-pairs modes; the device-only variant;
and the device rows handed out by i2_mesh_device_pairs."""
import numpy as np
import pytest

from tests._util import ensure_built

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    ensure_built()
    from integrator2_gb300 import api as A
    return A


def _plane(n, seed):
    """an open, jittered n x n grid (boundary edges, valence 3..6)"""
    rng = np.random.default_rng(seed)
    x, y = np.meshgrid(np.arange(n + 1.0), np.arange(n + 1.0), indexing="ij")
    V = np.stack([x, y, 0.05 * rng.normal(size=x.shape)], -1).reshape(-1, 3)
    V[:, :2] += rng.uniform(-0.2, 0.2, size=(len(V), 2))
    idx = np.arange((n + 1) ** 2).reshape(n + 1, n + 1)
    a, b, c, d = idx[:-1, :-1], idx[1:, :-1], idx[1:, 1:], idx[:-1, 1:]
    C = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)])
    return V, C.astype(np.int32)


def _cases():
    from integrator2_gb300 import meshes
    out = [("jittered icosphere s3", *meshes.jittered_icosphere(3, 0.15, 5)),
           ("torus 120x40", *meshes.torus(120, 40, 1.0, 0.25, jitter_rel=0.05, seed=3)),
           ("ellipsoid with pole fans", *meshes.ellipsoid(24, 96, (1.0, 2.0, 0.5))),
           ("open plane", *_plane(40, 7)),
           ("icosphere at 5e-4", *meshes.jittered_icosphere(2, 0.1, 9, 5e-4))]
    for V, C, kind, scale in meshes.uneven_mesh_set(11, 3, 500, 3000):
        out.append((f"uneven {kind} x{scale:.3g}", V, C))
    return out


def _lists(m):
    return [m.getSimpleNeighbors(), m.getAttachedNeighbors(), m.getNotNeighbors(), m.getSelfPairs()]


@pytest.mark.parametrize("near", [3.0, 1.5, None])
def test_device_builder_matches_host_builder(api, near):
    for name, V, C in _cases():
        if near is None and len(C) > 4000:
            continue
        h = api.Mesh3D()
        h.setGeometry(V, C)
        h.prepareMesh(near)
        d = api.Mesh3D()
        d.setGeometry(V, C)
        d.prepareMeshDevice(near)
        for cls, (a, b) in enumerate(zip(_lists(h), _lists(d))):
            assert a.shape == b.shape and np.array_equal(a, b), (name, near, cls, a.shape, b.shape)
        assert len(_lists(h)[2]) > 0 or near is not None, name


def test_device_only_lists_and_device_rows(api):
    import torch
    from integrator2_gb300 import meshes

    class Rows:
        def __init__(self, ptr, n):
            self.__cuda_array_interface__ = {"shape": (n, 2), "typestr": "<i4", "data": (ptr, False), "version": 3}

    V, C = meshes.torus(200, 50, 1.0, 0.2, jitter_rel=0.05, seed=1)
    h = api.Mesh3D()
    h.setGeometry(V, C)
    h.prepareMesh(3.0)
    d = api.Mesh3D()
    d.setGeometry(V, C)
    d.prepareMeshDevice(3.0, host_copy=False)
    for cls in range(4):
        ptr, n = d.devicePairs(cls)
        ref = _lists(h)[cls][:, :2]
        assert n == len(ref)
        got = torch.as_tensor(Rows(ptr, n), device="cuda").cpu().numpy()
        assert np.array_equal(got, ref), cls
        # a host-prepared mesh uploads its lists on request
        ptr2, n2 = h.devicePairs(cls)
        assert n2 == n and np.array_equal(torch.as_tensor(Rows(ptr2, n2), device="cuda").cpu().numpy(), ref)
    # host-side calls fetch the device-only lists
    for a, b in zip(_lists(h), _lists(d)):
        assert np.array_equal(a, b)


def test_device_rows_drive_the_evaluator(api):
    """the ordered (i, j) + (j, i) rows built on the device from the device lists give the same
    results as the host-built lists run through the host entry point"""
    import torch
    from integrator2_gb300 import meshes

    class Rows:
        def __init__(self, ptr, n):
            self.__cuda_array_interface__ = {"shape": (n, 2), "typestr": "<i4", "data": (ptr, False), "version": 3}

    V, C = meshes.jittered_icosphere(2, 0.15, 4)
    m = api.Mesh3D()
    m.setGeometry(V, C)
    m.prepareMeshDevice(3.0, host_copy=False)
    it = api.NumericalIntegrator3D(m, api.qf3D13)
    it.setErrorControl(api.RELATIVE_ERROR_CONTROL, 1e-6, 5)
    ev = api.EvaluatorJ3DK(m, it)
    for cls in range(3):
        ptr, n = m.devicePairs(cls)
        u = torch.as_tensor(Rows(ptr, n), device="cuda")
        rows = torch.cat([u, u.flip(1)]).contiguous()
        J = torch.empty(len(rows), 3, dtype=torch.float64, device="cuda")
        P = torch.empty(len(rows), dtype=torch.float64, device="cuda")
        ev.runClassDevice(cls, rows.data_ptr(), len(rows), 0, J.data_ptr(), P.data_ptr())
        ev.synchronize()
        ev2 = api.EvaluatorJ3DK(m, it)
        ev2.runClass(cls, rows.cpu().numpy())
        assert np.array_equal(J.cpu().numpy(), ev2.getResults(cls)), cls
