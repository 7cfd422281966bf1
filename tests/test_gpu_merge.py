"""The merge pass on the GPU (cuacd_merge_hulls, csrc/decompose.cpp) — the
reference's tests/merge.test.ts:33-76 ported, and the whole pass against the
oracle's restatement of src/merge.ts:170-303 (oracle/merge_oracle.cpp).

Against the oracle: the same number of parts, each output part holding the
same input parts in the same concatenation order (its mesh is bit for bit
their concatenation), the same mesh volume, hull volume within 1e-6
relative, the same seam count, Hausdorff within 1e-4 + 1e-3 d, and the same
statistics (rounds, merges, pairs hulled, pairs with a Hausdorff distance).
The merged hull meshes differ in triangulation: the engine cleans them with
its CPU quickhull as merge.ts:213 does, the oracle keeps the raw grid hull
faces, so the two passes sample different points of the same hull surface
and their Hausdorff distances agree to 1e-4 + 1e-2 d only. Each merged
part's Hausdorff distance is therefore also recomputed by the oracle on the
engine's own inputs — the part's mesh without the triangles on its seams
(filteredConcat) against its merged hull — and must agree to the GPU form's
1e-5 + 1e-4 d."""
import numpy as np
import pytest

import merge_cases as MC
from conftest import pkg

pytestmark = pytest.mark.gpu

D = pkg("decompose")
M = pkg("mesh")
G = pkg("meshgen")

# the reference merge test's tree (merge.test.ts:14)
SMALL = dict(vertexCap=4 << 20, triCap=4 << 20, edgeCap=1 << 18, scratchWords=4 << 20, hullBudgetBytes=32 << 20,
             hullMaxVerts=1024)


def _merge(parts, **kw):
    d = D.Decomposer(threshold=kw.get("threshold", 0.05), width=3, width2=3, tree=SMALL)
    try:
        return d.merge_hulls(parts, **kw)
    finally:
        d.destroy()


def test_merge_cube_halves_become_one_part():
    # merge.test.ts:33-48
    parts, st = _merge(MC.slabs([0.5]), threshold=0.05)
    assert len(parts) == 1
    p = parts[0]
    assert abs(p.meshVol - 1) < 1e-6 and abs(p.hullVol - 1) < 1e-5
    assert max(pkg("part").rv_cost(p.meshVol, p.hullVol), p.hausdorff or 0) < 0.01
    assert M.is_closed(p.mesh)
    assert len(p.seams) == 1 and p.merged == 2
    assert st["merges"] == 1 and st["rounds"] == 1


def test_merge_l_boxes_stay_apart():
    # merge.test.ts:56-63
    parts, st = _merge(MC.l_boxes(), threshold=0.05)
    assert len(parts) == 2
    assert st["pairsHulled"] == 1 and st["merges"] == 0


def test_merge_four_slabs_take_two_rounds():
    # merge.test.ts:65-76
    parts, st = _merge(MC.slabs([0.25, 0.5, 0.75]), threshold=0.05)
    assert len(parts) == 1
    assert st["rounds"] == 2 and st["merges"] == 3
    assert abs(parts[0].meshVol - 1) < 1e-6
    assert len(parts[0].seams) == 3
    one, _ = _merge(MC.slabs([0.25, 0.5, 0.75]), threshold=0.05, max_rounds=1)
    assert len(one) == 2


def _cases():
    return {
        "cube_halves": MC.slabs([0.5]),
        "four_slabs": MC.slabs([0.25, 0.5, 0.75]),
        "l_boxes": MC.l_boxes(),
        "grid_boxes": MC.grid_boxes(),
        "staircase_pieces": MC.cut_parts(G.staircase(8), [[0, 1, 0, -1.0], [0, 0, 1, -0.5], [1, 0, 0, -0.5]]),
        "sphere_pieces": MC.cut_parts(G.noisy_icosphere(2, noise=0.0, seed=3),
                                      [[1, 0, 0, -0.5], [0, 1, 0, -0.5], [0, 0, 1, -0.5]]),
    }


@pytest.mark.parametrize("name", list(_cases()))
def test_merge_matches_oracle(oracle, name):
    parts = _cases()[name]
    for thr in (0.05, 0.2):
        got, st = _merge(parts, threshold=thr)
        ref, rst = oracle.merge_hulls(parts, threshold=float(np.float32(thr)))
        assert len(got) == len(ref), (name, thr)
        for g, r in zip(got, ref):
            mem = r["members"]
            cat = parts[mem[0]].mesh
            for k in mem[1:]:
                cat = M.merge_meshes(cat, parts[k].mesh)
            assert np.array_equal(g.mesh.verts, cat.verts) and np.array_equal(g.mesh.tris, cat.tris), (name, thr, mem)
            assert g.meshVol == r["meshVol"]
            assert abs(g.hullVol - r["hullVol"]) <= 1e-6 * abs(r["hullVol"]) + 1e-12
            assert len(g.seams) == r["nSeams"] and g.merged == len(mem)
            if len(mem) > 1:
                d = r["hausdorff"]
                assert abs(g.hausdorff - d) <= 1e-4 + 1e-2 * d, (name, thr, g.hausdorff, d)
                empty = M.Mesh(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
                kept = oracle.filtered_concat(g.mesh, empty, g.seams, 1e-3)
                if len(kept) == 0:
                    assert g.hausdorff == 0.0
                else:
                    e = float(oracle.hausdorff_gpu_form([(M.Mesh(g.mesh.verts, kept), g.hull)])[0])
                    assert abs(g.hausdorff - e) <= 1e-5 + 1e-4 * e, (name, thr, g.hausdorff, e)
        for k in ("rounds", "merges", "pairsHulled", "pairsHausdorff"):
            assert st[k] == rst[k], (name, thr, k, st, rst)
