"""Errors of the GPU volumes, rv costs and Hausdorff distances stated against
FP64 references (and the Hausdorff screen against the FP32-only form).

FP64 references: mesh volumes by the divergence theorem summed exactly
(math.fsum of the float64 terms), hull volumes by qhull in double
(scipy.spatial.ConvexHull of the same float32 points), rv from those, and the
Hausdorff distance by the oracle's restatement of src/cpu/hausdorff.ts (the
same sampling rule, double arithmetic, exact nearest triangle through a BVH).

The bounds asserted are the stated precision of each quantity:
  tree child meshVol        5e-7 of the seed's volume absolute (float32
                            flux terms, compensated sums: the error does
                            not shrink with the part, so slivers show larger
                            relative errors), and 1e-5 relative for children
                            of at least 5 % of the seed's volume
  tree child hullVol        4e-6 relative (the hull's 2^21 integer grid)
  rv from tree volumes      2e-5 absolute
  cut half volume           1e-9 relative (fixed-order double sum)
  Hausdorff, screen on      1e-4 + 1e-3 d against FP64 (the reference's
                            GPU-vs-CPU tolerance, cpu.test.ts:97-111) and
                            1e-5 + 1e-4 d against the FP32-only form
Each test prints the largest errors it measured."""
import math

import numpy as np
import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu

G = pkg("meshgen")
M = pkg("mesh")
T = pkg("tree")
D = pkg("decompose")
P = pkg("part")


def vol64(m):
    """Signed volume in float64, summed exactly (the divergence theorem
    anchored at the origin)."""
    v = m.verts.astype(np.float64)
    a, b, c = v[m.tris[:, 0]], v[m.tris[:, 1]], v[m.tris[:, 2]]
    terms = np.einsum("ij,ij->i", a, np.cross(b, c))
    return math.fsum(terms.tolist()) / 6.0


def hull64(points):
    sp = pytest.importorskip("scipy.spatial")
    return float(sp.ConvexHull(np.asarray(points, np.float64)).volume)


def vol64_anchored(m, plane):
    """Volume of an uncapped half whose open rim lies in `plane`: the
    divergence theorem anchored at a point of the plane, where the missing
    cap's flux is zero, summed exactly in float64."""
    n = np.asarray(plane[:3], np.float64)
    o = -plane[3] * n / float(n @ n)
    v = m.verts.astype(np.float64) - o
    a, b, c = v[m.tris[:, 0]], v[m.tris[:, 1]], v[m.tris[:, 2]]
    return abs(math.fsum(np.einsum("ij,ij->i", a, np.cross(b, c)).tolist()) / 6.0)


def test_tree_volumes_and_rv_against_fp64():
    """Level-0 children of a tree run (depth 2, so they keep their
    triangles): each child's meshVol against the exact float64 volume of its
    own geometry, its hullVol against qhull of its own points."""
    seed = G.noisy_icosphere(3, noise=0.15, seed=5)
    g = T.GpuTree(width=6, width2=3, depth=2, nConcaveEdges=16, hullMaxVerts=4096)
    planes = G.random_planes(seed, 64, seed=7)
    g.run([seed], [planes])
    n_jobs = 6 + g.plane_slots
    jobs = g.jobs(0, n_jobs)
    errs = dict(meshVolAbs=0.0, meshVolRel=0.0, meshVolRelLarge=0.0, hullVol=0.0, rv=0.0)
    seed_vol = abs(M.signed_volume(seed))
    n = 0
    for j in range(n_jobs):
        if jobs[j, 6] != 1:  # valid after plan
            continue
        plane = jobs[j, 0:4].view(np.float32).astype(np.float64)
        for kid in (g.read_part(1 + 2 * j), g.read_part(1 + 2 * j + 1)):
            if kid["mesh"].nt == 0 or kid["mesh"].nv < 4:
                continue
            v64 = vol64_anchored(kid["mesh"], plane)
            h64 = hull64(kid["mesh"].verts)
            err = abs(kid["meshVol"] - v64)
            errs["meshVolAbs"] = max(errs["meshVolAbs"], err / seed_vol)
            errs["meshVolRel"] = max(errs["meshVolRel"], err / v64)
            if v64 >= 0.05 * seed_vol:
                errs["meshVolRelLarge"] = max(errs["meshVolRelLarge"], err / v64)
            errs["hullVol"] = max(errs["hullVol"], abs(kid["hullVol"] - h64) / h64)
            errs["rv"] = max(errs["rv"], abs(P.rv_cost(kid["meshVol"], kid["hullVol"]) - P.rv_cost(v64, h64)))
            n += 1
    print(f"tree level-0 children vs FP64 ({n} parts; meshVolAbs relative to the seed's volume): {errs}")
    assert n >= 40
    assert errs["meshVolAbs"] <= 5e-7 and errs["meshVolRelLarge"] <= 1e-5
    assert errs["hullVol"] <= 4e-6 and errs["rv"] <= 2e-5


def test_cut_evaluation_against_fp64(oracle):
    """The icosphere configuration's halves: volumes, hull volumes, rv and
    Hausdorff distances of cuacd_tree_eval_cuts against FP64."""
    m = G.noisy_icosphere(4, noise=0.15, seed=0)
    planes = G.random_planes(m, 16, seed=0).astype(np.float64)
    g = T.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096, scratchWords=64 << 20)
    got = g.eval_cuts(m, planes)
    cuts = g.plane_cuts([m], planes, np.zeros(len(planes), np.int32), closed=True)
    errs = dict(meshVol=0.0, hullVol=0.0, rv=0.0, hd64=0.0, hd32=0.0)
    for k, (st, pos, neg) in enumerate(cuts):
        assert (st == 0) == (got[k, 0] == 1)
        if st != 0:
            continue
        hd64 = 0.0
        for s, half in enumerate((pos, neg)):
            v64 = abs(vol64(half))
            h64 = hull64(half.verts)
            errs["meshVol"] = max(errs["meshVol"], abs(got[k, 1 + s] - v64) / v64)
            errs["hullVol"] = max(errs["hullVol"], abs(got[k, 3 + s] - h64) / h64)
            errs["rv"] = max(errs["rv"], abs(got[k, 5 + s] - P.rv_cost(v64, h64)))
            hull, _ = g.hull_meshes([half])
            hm = M.Mesh(half.verts, hull[0]["tris"])
            hd64 = max(hd64, oracle.hausdorff_cpu(half, hm))
        d = got[k, 7]
        errs["hd64"] = max(errs["hd64"], abs(d - hd64) / (1e-4 + 1e-3 * hd64))
    print(f"cut halves vs FP64 (errors; Hausdorff as a fraction of its tolerance): {errs}")
    assert errs["meshVol"] <= 1e-9 and errs["hullVol"] <= 4e-6 and errs["rv"] <= 2e-5 and errs["hd64"] <= 1.0


def test_hausdorff_screen_against_fp32_and_fp64(oracle):
    """The tensor-core screen (targets of >= 256 triangles) is bit-identical
    to the exhaustive FP32 search and within the stated tolerances of the
    FP32-only and FP64 forms, also for meshes far from the origin, where
    |p|^2 and -2 p.c cancel and the screen's error bound keeps every
    triangle (it then prunes nothing but stays exact)."""
    base = [G.noisy_icosphere(4, seed=s) for s in (1, 2)] + [M.normalize(G.blob_mesh(12, 40, seed=4))[0]]
    meshes = []
    for off in ((0, 0, 0), (1000.0, -500.0, 250.0)):
        for m in base:
            meshes.append(M.Mesh((m.verts.astype(np.float64) + off).astype(np.float32), m.tris))
    g = T.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096, scratchWords=256 << 20)
    hulls, _ = g.hull_meshes(meshes)
    pairs = [(m, M.Mesh(m.verts, h["tris"])) for m, h in zip(meshes, hulls)]
    screened = g.hausdorff(pairs)
    st = g.hd_stats()
    ex = T.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096, scratchWords=256 << 20,
                   hdScreenMinTris=-1).hausdorff(pairs)
    assert st["screened"] > 0 and not st["timeout"]
    assert np.array_equal(screened.view(np.uint32), ex.view(np.uint32))
    f32 = oracle.hausdorff_gpu_form(pairs)
    e32 = e64 = 0.0
    for k, (a, b) in enumerate(pairs):
        d32 = float(f32[k])
        d64 = oracle.hausdorff_cpu(a, b)
        e32 = max(e32, abs(screened[k] - d32) / (1e-5 + 1e-4 * d32))
        e64 = max(e64, abs(screened[k] - d64) / (1e-4 + 1e-3 * d64))
    print(f"Hausdorff screen: {st['exact']} of {st['screened']} screened pairs exact; error as a fraction of the "
          f"tolerance: FP32 form {e32:.3g}, FP64 form {e64:.3g}")
    assert e32 <= 1.0 and e64 <= 1.0
