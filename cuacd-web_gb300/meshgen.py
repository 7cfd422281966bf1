"""Seeded synthetic meshes for the benchmark workloads.

* ``icosphere`` / ``noisy_icosphere``: subdivided icosahedron, optionally
  displaced radially by seeded uniform noise and normalised to the unit cube.
* ``staircase``: the union of n axis-aligned boxes (width 1, depth 0.25,
  heights k * 0.125), welded into one closed manifold.
* ``random_planes``: seeded candidate planes through a mesh.
* ``blob_mesh``: an isosurface of a sum of Gaussian blobs, meshed by marching
  tetrahedra (see ``isosurface``).
"""
from __future__ import annotations

import numpy as np

from .mesh import Mesh


def icosphere(level: int) -> Mesh:
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(level):
        cache = {}

        def mid(a, b):
            k = (min(a, b), max(a, b))
            if k not in cache:
                p = verts[a] + verts[b]
                verts.append(p / np.linalg.norm(p))
                cache[k] = len(verts) - 1
            return cache[k]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return Mesh(np.array(verts, np.float32), np.array(faces, np.uint32))


def noisy_icosphere(level: int = 4, noise: float = 0.15, seed: int = 0) -> Mesh:
    """Icosphere with every vertex displaced radially by U[-noise, noise] of
    the radius, then uniformly scaled into the unit cube [0, 1]^3."""
    m = icosphere(level)
    rng = np.random.default_rng(seed)
    v = m.verts.astype(np.float64)
    v = v * (1.0 + rng.uniform(-noise, noise, size=(len(v), 1)))
    lo, hi = v.min(0), v.max(0)
    v = (v - lo) / (hi - lo).max()
    return Mesh(v.astype(np.float32), m.tris)


def random_planes(m: Mesh, n: int, seed: int = 0) -> np.ndarray:
    """n planes (a, b, c, d) with unit normals uniform on the sphere and
    offsets uniform over the mesh's extent along each normal."""
    rng = np.random.default_rng(seed)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    proj = m.verts.astype(np.float64) @ nrm.T  # (nv, n)
    lo, hi = proj.min(0), proj.max(0)
    off = lo + rng.uniform(0.0, 1.0, size=n) * (hi - lo)
    return np.concatenate([nrm, -off[:, None]], axis=1).astype(np.float32)


def staircase(n_steps: int = 8, width: float = 1.0, depth: float = 0.25, rise: float = 0.125) -> Mesh:
    """Union of n_steps boxes [0, width] x [(k-1) depth, k depth] x [0, k rise],
    k = 1..n_steps, as one closed manifold without T-junctions.

    Each side wall (x = 0 and x = width) is split into one polygon per box
    column: a quad for the first column and a pentagon (the previous
    column's top corner on its left edge) for the others, fanned from the
    bottom-left corner. Treads, risers, the back wall and the bottom are one
    quad per box. For n_steps = 8 this is 96 triangles.
    """
    ys = [k * depth for k in range(n_steps + 1)]
    hs = [k * rise for k in range(n_steps + 1)]
    verts = []
    index = {}

    def vid(x, y, z):
        key = (round(x, 9), round(y, 9), round(z, 9))
        if key not in index:
            index[key] = len(verts)
            verts.append((x, y, z))
        return index[key]

    tris = []

    def quad(a, b, c, d):  # counter-clockwise seen from outside
        tris.extend([(a, b, c), (a, c, d)])

    for side, x in ((0, 0.0), (1, width)):
        for k in range(1, n_steps + 1):
            y0, y1, h = ys[k - 1], ys[k], hs[k]
            poly = [(y0, 0.0), (y1, 0.0), (y1, h), (y0, h)]
            if k > 1:
                poly.append((y0, hs[k - 1]))
            ids = [vid(x, y, z) for y, z in poly]
            # outward normal of the x = 0 wall is -x: the (y, z) polygon above
            # is counter-clockwise seen from +x, so wall 0 is reversed
            for i in range(1, len(ids) - 1):
                t = (ids[0], ids[i], ids[i + 1])
                tris.append(t if side == 1 else (t[0], t[2], t[1]))
    for k in range(1, n_steps + 1):
        y0, y1, h = ys[k - 1], ys[k], hs[k]
        # tread (+z)
        quad(vid(0, y0, h), vid(width, y0, h), vid(width, y1, h), vid(0, y1, h))
        # riser facing -y, from the previous tread (or the floor) up to h
        hp = hs[k - 1]
        quad(vid(0, y0, hp), vid(width, y0, hp), vid(width, y0, h), vid(0, y0, h))
        # bottom (-z)
        quad(vid(0, y0, 0), vid(0, y1, 0), vid(width, y1, 0), vid(width, y0, 0))
    # back wall (+y) at y = n_steps * depth
    yb, hb = ys[-1], hs[-1]
    quad(vid(0, yb, 0), vid(0, yb, hb), vid(width, yb, hb), vid(width, yb, 0))
    return _orient_outward(Mesh(np.array(verts, np.float32), np.array(tris, np.uint32)))


def _orient_outward(m: Mesh) -> Mesh:
    from .mesh import signed_volume

    if signed_volume(m) < 0:
        return Mesh(m.verts, m.tris[:, [0, 2, 1]])
    return m
