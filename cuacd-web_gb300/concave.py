"""Candidate cutting planes from concave mesh edges (the reference's
src/cpu/concave.ts:25-92): the tree's edge-plane input.

For every undirected edge (v0 < v1, in ascending vertex order) whose dihedral
angle exceeds ``concave_threshold``, a deterministic reservoir of
``n_concave_edges`` edges is kept (the reference's LCG, seed 12345 unless
given); each kept edge yields two face-offset planes and, when the normals are
not nearly opposite, two bisector planes offset by +-eps.

The planes come from the library (``cuacd_concave_planes``), the one
implementation the decomposer also uses; this module only adds the
refinement spacing of the tree's probe rounds.
"""
from __future__ import annotations

import numpy as np

from .mesh import Mesh


def concave_edge_planes(m: Mesh, n_concave_edges: int = 16, concave_eps: float = 0.005,
                        concave_threshold: float = 3.49, seed: int = 12345) -> np.ndarray:
    """Planes (a, b, c, d) as a float32 array of shape (k, 4)."""
    if n_concave_edges <= 0 or m.nt == 0:
        return np.zeros((0, 4), np.float32)
    from .decompose import concave_planes

    return concave_planes(m, n_concave_edges, concave_eps, concave_threshold, seed)


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
