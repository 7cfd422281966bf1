"""Candidate cutting planes from concave mesh edges (the reference's
src/cpu/concave.ts:25-92): the tree's edge-plane input.

For every undirected edge (v0 < v1, in ascending vertex order) whose dihedral
angle exceeds ``concave_threshold``, a deterministic reservoir of
``n_concave_edges`` edges is kept (the reference's LCG, seed 12345 unless
given); each kept edge yields two face-offset planes and, when the normals are
not nearly opposite, two bisector planes offset by +-eps.
"""
from __future__ import annotations

import math

import numpy as np

from .mesh import Mesh


def _face_normals(v: np.ndarray, t: np.ndarray):
    a, b, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    n = np.cross(b - a, c - a)
    ln = np.linalg.norm(n, axis=1)
    ok = ln >= 1e-12
    n = np.where(ok[:, None], n / np.where(ok, ln, 1.0)[:, None], 0.0)
    return n, ok


def concave_edge_planes(m: Mesh, n_concave_edges: int = 16, concave_eps: float = 0.005,
                        concave_threshold: float = 3.49, seed: int = 12345) -> np.ndarray:
    """Planes (a, b, c, d) as a float32 array of shape (k, 4)."""
    if n_concave_edges <= 0 or m.nt == 0:
        return np.zeros((0, 4), np.float32)
    v = m.verts.astype(np.float64)
    t = m.tris.astype(np.int64)
    nrm, nok = _face_normals(v, t)
    nt = len(t)
    src = t.reshape(-1)
    dst = t[:, [1, 2, 0]].reshape(-1)
    face = np.repeat(np.arange(nt), 3)
    # first face of each directed edge, in CSR order (edgeCSR, mesh.ts:82-94)
    key = src * m.nv + dst
    order = np.lexsort((np.arange(len(key)), key))
    ks = key[order]
    first = np.ones(len(ks), bool)
    first[1:] = ks[1:] != ks[:-1]
    face_of = dict(zip(ks[first].tolist(), face[order][first].tolist()))
    # undirected edges v0 < v1 in (v0, v1) order
    und = np.unique(np.stack([np.minimum(src, dst), np.maximum(src, dst)], 1), axis=0)
    rng = seed & 0xFFFFFFFF

    def lcg():
        nonlocal rng
        rng = (rng * 1664525 + 1013904223) & 0xFFFFFFFF
        return rng

    reservoir = []
    seen = 0
    for v0, v1 in und.tolist():
        fa = face_of.get(v0 * m.nv + v1)
        fb = face_of.get(v1 * m.nv + v0)
        if fa is None or fb is None:
            continue
        f0, f1 = min(fa, fb), max(fa, fb)
        if not (nok[f0] and nok[f1]):
            continue
        n0, n1 = nrm[f0], nrm[f1]
        cos_a = max(-1.0, min(1.0, float(n0 @ n1)))
        alpha = math.acos(cos_a)
        tri0 = t[f0]
        others = [int(x) for x in tri0 if x != v0 and x != v1]
        if not others:
            continue
        d = float((v[others[0]] - v[v0]) @ n1)
        dihedral = math.pi + alpha if d > 0 else math.pi - alpha
        if not dihedral > concave_threshold:
            continue
        seen += 1
        if len(reservoir) < n_concave_edges:
            reservoir.append((v0, v1, f0, f1))
        else:
            r = lcg()
            thresh = math.floor(n_concave_edges / seen * 4294967295)
            if r < thresh:
                reservoir[lcg() % n_concave_edges] = (v0, v1, f0, f1)
    out = []
    for v0, v1, f0, f1 in reservoir:
        n0, n1 = nrm[f0], nrm[f1]
        mid = (v[v0] + v[v1]) / 2
        out.append([*n1, -(n1 @ mid + concave_eps)])
        out.append([*n0, -(n0 @ mid + concave_eps)])
        b = n0 + n1
        bl = np.linalg.norm(b)
        if bl >= 1e-4:
            b = b / bl
            out.append([*b, -(b @ mid + concave_eps)])
            out.append([*b, -(b @ mid - concave_eps)])
    return np.asarray(out, np.float32).reshape(-1, 4)


def refine_spacing(meshes, threshold: float, width: int):
    """Initial half-width of the refinement scan per part: the level-0 grid
    spacing of its smallest axis (decompose.ts:199-212)."""
    min_edge = min(threshold / 4, 0.015)
    cpa = max(1, width // 3)
    out = []
    for m in meshes:
        ext = m.verts.max(0).astype(np.float64) - m.verts.min(0).astype(np.float64)
        valid = ext - 2 * min_edge
        s = [x / (cpa + 1) for x in valid if x > 0]
        out.append(min(s) if s else 0.0)
    return out
