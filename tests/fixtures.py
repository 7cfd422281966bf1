"""Fixture meshes of the reference's test suite (tests/fixtures.ts:4-77),
restated for pytest."""
from __future__ import annotations

import importlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
M = importlib.import_module("cuacd-web_gb300.mesh")
Mesh = M.Mesh


def square_torus() -> Mesh:
    """Outer half-width 1, inner 0.5, height 0.5; volume 1.5 (fixtures.ts:4-21)."""
    R, r, h = 1.0, 0.5, 0.25
    verts = []
    for s, z in ((R, -h), (R, h), (r, -h), (r, h)):
        verts += [(-s, -s, z), (s, -s, z), (s, s, z), (-s, s, z)]
    tris = []

    def quad(a, b, c, d):
        tris.extend([(a, b, c), (a, c, d)])

    for i in range(4):
        j = (i + 1) % 4
        quad(i, j, 4 + j, 4 + i)
        quad(8 + j, 8 + i, 12 + i, 12 + j)
        quad(4 + i, 4 + j, 12 + j, 12 + i)
        quad(j, i, 8 + i, 8 + j)
    return Mesh(np.array(verts, np.float32), np.array(tris, np.uint32))


def extrude_polygon(poly, height) -> Mesh:
    """Extrude a simple CCW polygon along +z (fixtures.ts:29-61)."""
    n = len(poly)
    verts = [(x, y, z) for z in (0.0, height) for x, y in poly]
    tris = []
    idx = list(range(n))

    def area2(a, b, c):
        return (poly[b][0] - poly[a][0]) * (poly[c][1] - poly[a][1]) - (poly[b][1] - poly[a][1]) * (poly[c][0] - poly[a][0])

    def inside(p, a, b, c):
        return area2(a, b, p) >= 0 and area2(b, c, p) >= 0 and area2(c, a, p) >= 0

    guard = 0
    while len(idx) > 3 and guard < 1000:
        guard += 1
        clipped = False
        for i in range(len(idx)):
            a, b, c = idx[(i + len(idx) - 1) % len(idx)], idx[i], idx[(i + 1) % len(idx)]
            if area2(a, b, c) <= 0:
                continue
            if any(p not in (a, b, c) and inside(p, a, b, c) for p in idx):
                continue
            tris.append((a, c, b))
            tris.append((n + a, n + b, n + c))
            idx.pop(i)
            clipped = True
            break
        if not clipped:
            break
    tris.append((idx[0], idx[2], idx[1]))
    tris.append((n + idx[0], n + idx[1], n + idx[2]))
    for i in range(n):
        j = (i + 1) % n
        tris.append((i, j, n + j))
        tris.append((i, n + j, n + i))
    return Mesh(np.array(verts, np.float32), np.array(tris, np.uint32))


def stairs() -> Mesh:
    """Welded 3-step prism, volume 6 (fixtures.ts:24-26)."""
    return extrude_polygon([(0, 0), (3, 0), (3, 1), (2, 1), (2, 2), (1, 2), (1, 3), (0, 3)], 1.0)


def l_prism() -> Mesh:
    """Welded L prism with one concave vertical edge (fixtures.ts:74-77)."""
    return extrude_polygon([(0, 0), (2, 0), (2, 1), (1, 1), (1, 2), (0, 2)], 1.0)
