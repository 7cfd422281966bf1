"""Triangle-mesh helpers (the reference's src/mesh.ts).

A :class:`Mesh` holds ``verts`` as a float32 array of shape (nv, 3) and
``tris`` as a uint32 array of shape (nt, 3), closed and outward wound.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Mesh:
    verts: np.ndarray  # (nv, 3) float32
    tris: np.ndarray  # (nt, 3) uint32

    def __post_init__(self):
        self.verts = np.ascontiguousarray(np.asarray(self.verts, dtype=np.float32).reshape(-1, 3))
        self.tris = np.ascontiguousarray(np.asarray(self.tris, dtype=np.uint32).reshape(-1, 3))

    @property
    def nv(self) -> int:
        return int(self.verts.shape[0])

    @property
    def nt(self) -> int:
        return int(self.tris.shape[0])


def make_box(lo, hi) -> Mesh:
    """Axis-aligned box (mesh.ts:20-38)."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    verts = [
        x0, y0, z0, x1, y0, z0, x1, y1, z0, x0, y1, z0,
        x0, y0, z1, x1, y0, z1, x1, y1, z1, x0, y1, z1,
    ]
    tris = [
        0, 2, 1, 0, 3, 2,
        4, 5, 6, 4, 6, 7,
        0, 1, 5, 0, 5, 4,
        2, 3, 7, 2, 7, 6,
        1, 2, 6, 1, 6, 5,
        0, 4, 7, 0, 7, 3,
    ]
    return Mesh(np.array(verts, np.float32), np.array(tris, np.uint32))


def merge_meshes(a: Mesh, b: Mesh) -> Mesh:
    """Concatenation of two meshes (mesh.ts:40-49)."""
    return Mesh(np.concatenate([a.verts, b.verts]), np.concatenate([a.tris, b.tris + a.nv]))


def unit_cube() -> Mesh:
    return make_box((0, 0, 0), (1, 1, 1))


def l_shape() -> Mesh:
    """Two boxes joined along x (mesh.ts:57-59); not welded."""
    return merge_meshes(make_box((0, 0, 0), (1, 1, 1)), make_box((1, 0, 0), (2, 1, 0.5)))


def signed_volume(m: Mesh) -> float:
    """Divergence-theorem volume anchored at vertex 0 (mesh.ts:61-75)."""
    if m.nt == 0:
        return 0.0
    v = m.verts.astype(np.float64) - m.verts[0].astype(np.float64)
    a, b, c = v[m.tris[:, 0]], v[m.tris[:, 1]], v[m.tris[:, 2]]
    return float(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0)


def volume(m: Mesh) -> float:
    return abs(signed_volume(m))


def is_closed(m: Mesh) -> bool:
    """Every directed edge occurs once and its reverse once (mesh.ts:96-110)."""
    if m.nt == 0:
        return False
    t = m.tris.astype(np.int64)
    if t.max() >= m.nv:
        return False
    src = t.reshape(-1)
    dst = t[:, [1, 2, 0]].reshape(-1)
    key = src * m.nv + dst
    u, cnt = np.unique(key, return_counts=True)
    if (cnt != 1).any():
        return False
    rev = dst * m.nv + src
    return bool(np.isin(rev, u, assume_unique=False).all())


def bbox(m: Mesh):
    return m.verts.min(axis=0), m.verts.max(axis=0)


def normalize(m: Mesh):
    """Center and scale the largest extent to 2 (mesh.ts:141-153).

    Returns the normalised mesh, the scale and the center.
    """
    lo, hi = bbox(m)
    center = (lo.astype(np.float64) + hi.astype(np.float64)) / 2
    extent = float((hi.astype(np.float64) - lo.astype(np.float64)).max())
    scale = extent / 2 if extent > 0 else 1.0
    verts = ((m.verts.astype(np.float64) - center) / scale).astype(np.float32)
    return Mesh(verts, m.tris.copy()), scale, center


def mesh_area(m: Mesh) -> float:
    v = m.verts.astype(np.float64)
    a, b, c = v[m.tris[:, 0]], v[m.tris[:, 1]], v[m.tris[:, 2]]
    return float(0.5 * np.linalg.norm(np.cross(b - a, c - a), axis=1).sum())
