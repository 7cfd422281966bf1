"""Decompositions of the reference's own test meshes on the GPU (the meshes
are committed under tests/golden/, copied from the reference's
tests/data/49160.stl and demo/models/{teapot,bunny}_vox64.stl.gz).

tests/decompose.test.ts:52-63: 49160.stl at maxIters 100, threshold 0.05,
width 30 on the small test tree: every part closed, the parts' volumes sum to
the mesh's within 1e-3 of it. The README's comparison settings (width 30,
nConcaveEdges 16, threshold 0.05, merging on; README.md:151-157) on the
teapot: the same checks. Parts and times are printed beside the reference's
(142 / 16 / 246 parts on an RTX 4090)."""
import gzip
import os

import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu

D = pkg("decompose")
M = pkg("mesh")
IO = pkg("meshio")
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SMALL = dict(vertexCap=4 << 20, triCap=4 << 20, edgeCap=1 << 18, scratchWords=4 << 20, hullBudgetBytes=32 << 20,
             hullMaxVerts=1024)
BIG = dict(vertexCap=256 << 20, triCap=256 << 20, edgeCap=16 << 20, scratchWords=256 << 20, hullBudgetBytes=16 << 30,
           hullMaxVerts=32768)


def load(name):
    with open(os.path.join(HERE, name), "rb") as f:
        buf = f.read()
    if name.endswith(".gz"):
        buf = gzip.decompress(buf)
    return IO.parse_stl(buf)


def _check(mesh, r):
    total = 0.0
    for p in r.parts:
        assert M.is_closed(p.mesh)
        total += M.volume(p.mesh)
    v = M.volume(mesh)
    assert abs(total - v) <= 1e-3 * v, (total, v)


def test_49160_converges_with_closed_parts():
    mesh = load("49160.stl")
    assert M.is_closed(mesh)
    r = D.decompose(mesh, maxIters=100, threshold=0.05, width=30, tree=SMALL)
    print(f"49160.stl: {len(r.parts)} parts in {r.iterations} iterations, {r.stats['totalMs']:.0f} ms")
    assert len(r.parts) >= 1
    _check(mesh, r)


def test_readme_settings_49160_and_teapot():
    for name in ("49160.stl", "teapot_vox64.stl.gz"):
        mesh = load(name)
        assert M.is_closed(mesh)
        r = D.decompose(mesh, threshold=0.05, width=30, nConcaveEdges=16, mergeHulls=True, tree=BIG)
        print(f"{name}: {mesh.nt} triangles, {len(r.parts)} parts in {r.iterations} iterations, "
              f"{r.stats['totalMs']:.0f} ms")
        _check(mesh, r)
