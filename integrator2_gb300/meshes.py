"""Synthetic surface meshes and the reference's ``.dat`` mesh format.

Every workload of this library is a closed triangulated surface (no public data set is
involved): icospheres, jittered icospheres, spherical-harmonic displaced spheres, ellipsoid
and torus grids.  All generators are seeded and return ``(vertices float64[nv,3],
cells int32[nc,3])`` with outward (counter-clockwise seen from outside) orientation, the
orientation the reference assumes for its vertex-class branch choices
(evaluatorJ3DK.cu:699-703).
"""
from __future__ import annotations

import math
from typing import Tuple

import numpy as np

Mesh = Tuple[np.ndarray, np.ndarray]

_PHI = (1.0 + 5.0 ** 0.5) / 2.0


def icosahedron() -> Mesh:
    v = np.array([[-1, _PHI, 0], [1, _PHI, 0], [-1, -_PHI, 0], [1, -_PHI, 0],
                  [0, -1, _PHI], [0, 1, _PHI], [0, -1, -_PHI], [0, 1, -_PHI],
                  [_PHI, 0, -1], [_PHI, 0, 1], [-_PHI, 0, -1], [-_PHI, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int32)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v, f


def subdivide(v: np.ndarray, f: np.ndarray, project: bool = True) -> Mesh:
    """One 1->4 midpoint subdivision with shared edge midpoints; optional unit-sphere projection."""
    nv = len(v)
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    key = np.minimum(e[:, 0], e[:, 1]).astype(np.int64) * (nv + 1) + np.maximum(e[:, 0], e[:, 1])
    uniq, inv = np.unique(key, return_inverse=True)
    a = (uniq // (nv + 1)).astype(np.int64)
    b = (uniq % (nv + 1)).astype(np.int64)
    mid = 0.5 * (v[a] + v[b])
    if project:
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
    m = (inv + nv).reshape(3, -1).T  # midpoints of edges (01, 12, 20) per face
    i0, i1, i2 = f[:, 0], f[:, 1], f[:, 2]
    m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
    nf = np.concatenate([np.stack([i0, m01, m20], 1), np.stack([i1, m12, m01], 1),
                         np.stack([i2, m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return np.concatenate([v, mid]), nf.astype(np.int32)


def icosphere(subdivisions: int, radius: float = 1.0) -> Mesh:
    v, f = icosahedron()
    for _ in range(subdivisions):
        v, f = subdivide(v, f)
    return radius * v, f


def geodesic_sphere(freq: int, radius: float = 1.0) -> Mesh:
    """Class-I geodesic sphere: every icosahedron face split into freq^2 triangles on a
    barycentric grid, projected to the sphere; 20 freq^2 cells, 10 freq^2 + 2 vertices, any
    freq >= 1 (the 1->4 icospheres are freq = 2^s).  A grid point a + i (b - a) / n + j (c - a) / n
    is keyed by its integer barycentric weights on the icosahedron's vertices, so points on an edge
    or corner shared by two faces are one vertex."""
    v0, f0 = icosahedron()
    n = int(freq)
    if n < 1:
        raise ValueError("freq must be >= 1")
    index, verts, cells = {}, [], []

    def vid(face, i, j):
        w = {face[0]: n - i - j, face[1]: i, face[2]: j}
        key = tuple(sorted((int(k), int(c)) for k, c in w.items() if c))
        if key not in index:
            p = sum(c * v0[k] for k, c in key) / n
            index[key] = len(verts)
            verts.append(p / np.linalg.norm(p))
        return index[key]

    for face in f0:
        for i in range(n):
            for j in range(n - i):
                cells.append((vid(face, i, j), vid(face, i + 1, j), vid(face, i, j + 1)))
                if i + j < n - 1:
                    cells.append((vid(face, i + 1, j), vid(face, i + 1, j + 1), vid(face, i, j + 1)))
    return radius * np.asarray(verts), np.asarray(cells, np.int32)


def tangential_jitter(v: np.ndarray, f: np.ndarray, sigma_rel: float, seed: int) -> np.ndarray:
    """vertices of a sphere mesh moved by a seeded Gaussian tangential jitter of sigma_rel x the
    mean edge length and reprojected to the sphere's radius"""
    r = np.linalg.norm(v, axis=1, keepdims=True)
    u = v / r
    h = mean_edge_length(u, f)
    rng = np.random.default_rng(seed)
    d = rng.normal(0.0, sigma_rel * h, size=v.shape)
    d -= np.sum(d * u, axis=1, keepdims=True) * u
    w = u + d
    return r * (w / np.linalg.norm(w, axis=1, keepdims=True))


def edge_lengths(v: np.ndarray, f: np.ndarray) -> np.ndarray:
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    e = np.unique(np.sort(e, axis=1), axis=0)
    return np.linalg.norm(v[e[:, 0]] - v[e[:, 1]], axis=1)


def mean_edge_length(v: np.ndarray, f: np.ndarray) -> float:
    return float(edge_lengths(v, f).mean())


def jittered_icosphere(subdivisions: int, sigma_rel: float, seed: int, radius: float = 1.0) -> Mesh:
    """Icosphere whose vertices get a seeded Gaussian tangential jitter of sigma_rel x mean edge
    length, then are reprojected to the sphere."""
    v, f = icosphere(subdivisions, 1.0)
    h = mean_edge_length(v, f)
    rng = np.random.default_rng(seed)
    d = rng.normal(0.0, sigma_rel * h, size=v.shape)
    d -= np.sum(d * v, axis=1, keepdims=True) * v          # tangential part
    w = v + d
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    return radius * w, f


def _real_sph_harm(l: int, m: int, theta: np.ndarray, phi: np.ndarray) -> np.ndarray:
    """Real spherical harmonic Y_lm (orthonormal), theta polar, phi azimuth."""
    from scipy.special import lpmv
    am = abs(m)
    norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
    p = lpmv(am, l, np.cos(theta))
    if m > 0:
        return math.sqrt(2.0) * norm * p * np.cos(am * phi)
    if m < 0:
        return math.sqrt(2.0) * norm * p * np.sin(am * phi)
    return norm * p


def sh_displaced_icosphere(subdivisions: int, lmax: int, amp: float, seed: int) -> Mesh:
    """Icosphere displaced radially by sum_{l<=lmax} a_lm Y_lm, a_lm ~ N(0, amp^2)."""
    v, f = icosphere(subdivisions, 1.0)
    rng = np.random.default_rng(seed)
    theta = np.arccos(np.clip(v[:, 2], -1, 1))
    phi = np.arctan2(v[:, 1], v[:, 0])
    r = np.ones(len(v))
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            r += rng.normal(0.0, amp) * _real_sph_harm(l, m, theta, phi)
    return v * r[:, None], f


def torus(n_major: int, n_minor: int, R: float = 1.0, r: float = 0.1, scale: float = 1.0,
          jitter_rel: float = 0.0, seed: int = 0) -> Mesh:
    """Torus grid triangulated into 2*n_major*n_minor cells, optional seeded normal jitter
    of jitter_rel x the local edge length."""
    u = 2 * np.pi * np.arange(n_major) / n_major
    w = 2 * np.pi * np.arange(n_minor) / n_minor
    U, W = np.meshgrid(u, w, indexing="ij")
    x = (R + r * np.cos(W)) * np.cos(U)
    y = (R + r * np.cos(W)) * np.sin(U)
    z = r * np.sin(W)
    v = np.stack([x, y, z], -1).reshape(-1, 3)
    idx = np.arange(n_major * n_minor).reshape(n_major, n_minor)
    a = idx
    b = np.roll(idx, -1, axis=0)
    c = np.roll(np.roll(idx, -1, axis=0), -1, axis=1)
    d = np.roll(idx, -1, axis=1)
    f = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)])
    if jitter_rel > 0:
        nrm = np.stack([np.cos(W) * np.cos(U), np.cos(W) * np.sin(U), np.sin(W)], -1).reshape(-1, 3)
        step = min(2 * np.pi * (R - r) / n_major, 2 * np.pi * r / n_minor)
        rng = np.random.default_rng(seed)
        v = v + nrm * rng.normal(0.0, jitter_rel * step, size=(len(v), 1))
    return scale * v, f.astype(np.int32)


def ellipsoid(n_theta: int, n_phi: int, axes=(1.0, 1.0, 1.0), scale: float = 1.0) -> Mesh:
    """Latitude-longitude ellipsoid grid with pole fans: 2*n_phi*(n_theta-1) cells."""
    th = np.pi * np.arange(1, n_theta) / n_theta
    ph = 2 * np.pi * np.arange(n_phi) / n_phi
    T, P = np.meshgrid(th, ph, indexing="ij")
    ring = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], -1).reshape(-1, 3)
    v = np.concatenate([[[0, 0, 1]], ring, [[0, 0, -1]]]) * np.asarray(axes)
    nr = n_theta - 1
    idx = 1 + np.arange(nr * n_phi).reshape(nr, n_phi)
    south = 1 + nr * n_phi
    faces = []
    for k in range(n_phi):
        k1 = (k + 1) % n_phi
        faces.append([0, idx[0, k], idx[0, k1]])
        faces.append([south, idx[nr - 1, k1], idx[nr - 1, k]])
    for i in range(nr - 1):
        for k in range(n_phi):
            k1 = (k + 1) % n_phi
            faces.append([idx[i, k], idx[i + 1, k], idx[i + 1, k1]])
            faces.append([idx[i, k], idx[i + 1, k1], idx[i, k1]])
    return scale * v, np.asarray(faces, dtype=np.int32)


def uneven_mesh_set(seed: int, count: int = 48, tri_min: int = 500, tri_max: int = 60000):
    """A seeded set of independent closed meshes of uneven size and scale (a many-mesh batch
    workload): ellipsoids with semi-axes uniform in [0.3, 3] (stretched geodesic spheres), tori
    with R/r uniform in [2, 6] and jittered geodesic spheres (sigma 0.15 h), in turn; triangle
    counts log-uniform in [tri_min, tri_max] (the nearest grid size inside that range: 20 n^2 for
    the spheres, 2 n_major n_minor for the tori); scales uniform in [5e-4, 1e2].
    Returns [(V, C, kind, scale)]."""
    rng = np.random.default_rng(seed)
    out = []
    f_lo, f_hi = math.ceil(math.sqrt(tri_min / 20.0)), math.floor(math.sqrt(tri_max / 20.0))
    for k in range(count):
        target = float(np.exp(rng.uniform(np.log(tri_min), np.log(tri_max))))
        scale = float(rng.uniform(5e-4, 1e2))
        kind = ("ellipsoid", "torus", "icosphere")[k % 3]
        freq = int(np.clip(round(math.sqrt(target / 20.0)), f_lo, f_hi))
        if kind == "ellipsoid":
            # a stretched geodesic sphere (a latitude-longitude grid would add pole fans of needles)
            axes = rng.uniform(0.3, 3.0, size=3)
            V, C = geodesic_sphere(freq, 1.0)
            V = scale * V * axes
        elif kind == "torus":
            ratio = rng.uniform(2.0, 6.0)
            n_minor = max(4, int(round(math.sqrt(target / (2.0 * ratio)))))
            cells = lambda m: 2 * int(round(ratio * m)) * m
            while cells(n_minor) > tri_max:
                n_minor -= 1
            while cells(n_minor) < tri_min:
                n_minor += 1
            V, C = torus(int(round(ratio * n_minor)), n_minor, 1.0, 1.0 / ratio, scale)
        else:
            V, C = geodesic_sphere(freq, 1.0)
            V = scale * tangential_jitter(V, C, 0.15, int(rng.integers(1 << 30)))
        out.append((V, C.astype(np.int32), kind, scale))
    return out


def orient_outward(v: np.ndarray, f: np.ndarray) -> np.ndarray:
    """Flip cells whose normal points towards the centroid of the surface (star-shaped meshes)."""
    c = v.mean(axis=0)
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    ctr = v[f].mean(axis=1)
    flip = np.sum(n * (ctr - c), axis=1) < 0
    g = f.copy()
    g[flip] = g[flip][:, [0, 2, 1]]
    return g


# ------------------------------------------------------------------------------- .dat I/O
def write_dat(path: str, v: np.ndarray, f: np.ndarray) -> None:
    """Reference mesh format: 'nv nc', then 'idx x y z' lines, then 'idx 203 a b c' (1-based)."""
    with open(path, "w") as fh:
        fh.write(f"{len(v)}\t{len(f)}\n")
        for k, p in enumerate(v):
            fh.write(f"{k + 1}\t{float(p[0])!r}\t{float(p[1])!r}\t{float(p[2])!r}\n")
        for k, c in enumerate(f):
            fh.write(f"{k + 1}\t203\t{c[0] + 1}\t{c[1] + 1}\t{c[2] + 1}\n")


def read_dat(path: str, scale: float = 1.0) -> Mesh:
    """Reads the reference's .dat format with the reference's semantics
    (src/Mesh3d.cu:159-217).  After the 'nv nc' header and nv 'idx x y z' lines come elements
    'idx type ...': type 203 is a triangle 'a b c' (1-based); any other type consumes two more
    tokens and lowers the cell count by one.  The kept cells are the first
    (header count - skipped elements) triangles in file order.  Trailing whitespace makes the
    reference's read loop turn once more on a failed read that leaves its last 'type' value in
    place: if that value was a triangle the extra turn changes nothing, otherwise it skips one
    more cell."""
    text = open(path).read()
    toks = text.split()
    nv, nc = int(toks[0]), int(toks[1])
    pos = 2
    v = np.empty((nv, 3))
    for k in range(nv):
        v[k] = [float(toks[pos + 1]), float(toks[pos + 2]), float(toks[pos + 3])]
        pos += 4
    cells = []
    last_type = 0
    while pos < len(toks):
        last_type = int(toks[pos + 1]) if pos + 1 < len(toks) else 0
        if last_type == 203:
            cells.append([int(toks[pos + 2]) - 1, int(toks[pos + 3]) - 1, int(toks[pos + 4]) - 1])
            pos += 5
        else:
            nc -= 1
            pos += 4
    if text[-1:].isspace() and last_type != 203:
        nc -= 1
    f = np.asarray(cells, dtype=np.int32).reshape(-1, 3)[:max(nc, 0)]
    return scale * v, f
