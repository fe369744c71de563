"""Ordered pair lists of the four pair classes.

The reference decides a pair's class by counting shared vertex indices over all i<j pairs
(src/Mesh3d.cu:93-142): 1 shared vertex = ``simple_neighbors`` (common vertex), 2 =
``attached_neighbors`` (common edge), 0 = ``not_neighbors`` (every disjoint pair).  This
module builds the same classes in O(N) from the cell-vertex incidence, adds the self class
(i, i) -- absent from the reference, which excludes i == j -- and restricts the disjoint class
to near-field pairs (centroid distance below ``near_factor`` x mean edge length) or, with
``near_factor=None``, keeps all disjoint pairs as the reference's runAllPairs does.

Lists are ordered pairs (both (i, j) and (j, i)), sorted i-major, as int32 arrays [n, 2].
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

VERTEX, EDGE, FAR, SELF = 0, 1, 2, 3
CLASS_NAMES = {VERTEX: "common-vertex", EDGE: "common-edge", FAR: "near-field", SELF: "self"}


@dataclass
class PairLists:
    vertex: np.ndarray
    edge: np.ndarray
    far: np.ndarray
    self_: np.ndarray

    def by_class(self, cls: int) -> np.ndarray:
        return {VERTEX: self.vertex, EDGE: self.edge, FAR: self.far, SELF: self.self_}[cls]

    def total(self) -> int:
        return len(self.vertex) + len(self.edge) + len(self.far) + len(self.self_)


def _shared_counts(f: np.ndarray):
    import scipy.sparse as sp
    nc = len(f)
    nv = int(f.max()) + 1
    rows = np.repeat(np.arange(nc), 3)
    inc = sp.csr_matrix((np.ones(3 * nc, dtype=np.int32), (rows, f.ravel())), shape=(nc, nv))
    shared = (inc @ inc.T).tocoo()
    return shared.row.astype(np.int64), shared.col.astype(np.int64), shared.data


def _sorted_pairs(i: np.ndarray, j: np.ndarray) -> np.ndarray:
    o = np.lexsort((j, i))
    return np.stack([i[o], j[o]], axis=1).astype(np.int32)


def build_pairs(v: np.ndarray, f: np.ndarray, near_factor: float | None = 3.0) -> PairLists:
    f = np.asarray(f, dtype=np.int64)
    r, c, d = _shared_counts(f)
    off = r != c
    vertex = _sorted_pairs(r[off & (d == 1)], c[off & (d == 1)])
    edge = _sorted_pairs(r[off & (d == 2)], c[off & (d == 2)])
    nc = len(f)
    self_ = np.stack([np.arange(nc), np.arange(nc)], axis=1).astype(np.int32)
    touching = set(zip(r[off].tolist(), c[off].tolist())) if nc <= 4096 else None
    if near_factor is None:
        ii, jj = np.meshgrid(np.arange(nc), np.arange(nc), indexing="ij")
        ii, jj = ii.ravel(), jj.ravel()
        keep = ii != jj
        ii, jj = ii[keep], jj[keep]
    else:
        from scipy.spatial import cKDTree
        from .meshes import mean_edge_length
        h = mean_edge_length(v, f)
        ctr = v[f].mean(axis=1)
        up = cKDTree(ctr).query_pairs(near_factor * h, output_type="ndarray")
        ii = np.concatenate([up[:, 0], up[:, 1]])
        jj = np.concatenate([up[:, 1], up[:, 0]])
    # drop pairs that share a vertex
    key_touch = np.unique(r[off] * nc + c[off]) if touching is None else None
    key = ii.astype(np.int64) * nc + jj
    if key_touch is not None:
        disjoint = ~np.isin(key, key_touch)
    else:
        tk = np.fromiter((a * nc + b for a, b in touching), dtype=np.int64, count=len(touching))
        disjoint = ~np.isin(key, tk)
    far = _sorted_pairs(ii[disjoint], jj[disjoint])
    return PairLists(vertex=vertex, edge=edge, far=far, self_=self_)
