"""Parity of the CUDA hull and Hausdorff batches (GpuTree.hullMeshes,
hausdorff, hullsWithHausdorff) with the CPU oracle, through the C ABI.

Hull face sets are compared exactly (same faces in the same order); volumes
to 1e-6 relative, and to the reference's own quickhull within the 2^21
grid's quantisation (3e-5). Hausdorff distances agree with the oracle's
float32 form within 1e-5 + 1e-4 d, and with the reference's CPU helper within
its own test tolerance, 1e-4 + 1e-3 d (tests/cpu.test.ts:97-111)."""
import importlib

import numpy as np
import pytest

from fixtures import M, l_prism, square_torus, stairs

pytestmark = pytest.mark.gpu
gen = importlib.import_module("cuacd-web_gb300.meshgen")


@pytest.fixture(scope="module")
def tree_mod():
    return importlib.import_module("cuacd-web_gb300.tree")


def point_sets():
    rng = np.random.default_rng(7)
    out = [
        M.unit_cube(), M.l_shape(), square_torus(), stairs(), gen.staircase(8), gen.noisy_icosphere(3, seed=1),
        M.Mesh(rng.normal(size=(500, 3)).astype(np.float32), np.zeros((0, 3), np.uint32)),
        M.Mesh(rng.uniform(-1, 1, size=(2000, 3)).astype(np.float32), np.zeros((0, 3), np.uint32)),
        # coplanar grid plus one apex: many exactly coplanar points
        M.Mesh(np.concatenate([np.stack(np.meshgrid(np.arange(8), np.arange(8), [0.0]), -1).reshape(-1, 3),
                               [[3.5, 3.5, 2.0]]]).astype(np.float32), np.zeros((0, 3), np.uint32)),
        # duplicated points
        M.Mesh(np.repeat(rng.normal(size=(40, 3)), 3, axis=0).astype(np.float32), np.zeros((0, 3), np.uint32)),
        # fewer than 4 points, and a flat set: no hull
        M.Mesh(np.eye(3, dtype=np.float32), np.zeros((0, 3), np.uint32)),
        M.Mesh(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [0.5, 0.5, 0]], np.float32), np.zeros((0, 3), np.uint32)),
    ]
    return out


def test_hull_faces_match_oracle(tree_mod, oracle):
    cfg = dict(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096)
    g = tree_mod.GpuTree(**cfg)
    o = oracle.OracleTree(**cfg)
    sets = point_sets()
    rg, sg = g.hull_meshes(sets)
    ro, so = o.hull_meshes(sets)
    assert list(sg) == list(so)
    for i, (a, b) in enumerate(zip(rg, ro)):
        assert (a is None) == (b is None), i
        if a is None:
            continue
        assert np.array_equal(a["tris"], b["tris"]), i
        assert np.float32(a["volume"]).view(np.uint32) == np.float32(b["volume"]).view(np.uint32), (i, a["volume"], b["volume"])
        h = M.Mesh(sets[i].verts, a["tris"])
        assert M.is_closed(h) and M.signed_volume(h) > 0, i
        if oracle.qh_ref_loaded():
            ref = oracle.hull_volume(sets[i], True)
            assert abs(a["volume"] - ref) <= 3e-5 * ref, (i, a["volume"], ref)


def test_hull_stages_and_large_parts(tree_mod, oracle):
    """Large point sets run on block groups; the staged variants of
    tests/bench_hull.ts stop early."""
    cfg = dict(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096)
    g = tree_mod.GpuTree(**cfg)
    o = oracle.OracleTree(**cfg)
    big = gen.noisy_icosphere(5, seed=2)  # 10242 points
    for stage in (0, 2):
        rg, sg = g.hull_meshes([big, big], hull_stage=stage)
        ro, so = o.hull_meshes([big, big], hull_stage=stage)
        assert list(sg) == list(so)
        for a, b in zip(rg, ro):
            assert (a is None) == (b is None)
            if a is not None:
                assert np.array_equal(a["tris"], b["tris"]) and a["volume"] == b["volume"]


def test_hull_compaction_heavy_sets(tree_mod, oracle):
    """Point sets whose hulls compact their face slots many times (every
    point on a sphere; a marching-tetrahedra blob whose vertices share grid
    lines and planes): after each compaction every candidate is reassigned
    over every face, which the kernel does by walking each point's visible
    patch."""
    cfg = dict(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096)
    g = tree_mod.GpuTree(**cfg)
    o = oracle.OracleTree(**cfg)
    rng = np.random.default_rng(11)
    s = rng.normal(size=(3000, 3))
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    inner = rng.uniform(-0.7, 0.7, size=(3000, 3))
    sets = [M.Mesh(np.concatenate([s, inner]).astype(np.float32), np.zeros((0, 3), np.uint32)),
            gen.blob_mesh(6, 26, seed=3)]
    rg, sg = g.hull_meshes(sets)
    ro, so = o.hull_meshes(sets)
    assert list(sg) == list(so)
    for a, b in zip(rg, ro):
        assert (a is None) == (b is None)
        if a is not None:
            assert np.array_equal(a["tris"], b["tris"]) and a["volume"] == b["volume"]


def test_hull_large_cut_parts(tree_mod, oracle):
    """Block-path hulls of large cut halves: a planar cap of many exactly
    coplanar points (axis-aligned cuts) on a curved surface whose vertices
    share grid lines, the shape of the large-mesh workload's parts."""
    D = importlib.import_module("cuacd-web_gb300.decompose")
    cfg = dict(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=16384)
    g = tree_mod.GpuTree(**cfg)
    o = oracle.OracleTree(**cfg)
    blob = M.normalize(gen.blob_mesh(12, 44, seed=4))[0]
    sets = []
    for pl in ([1, 0, 0, 0.1], [0, 1, 0, -0.05], [0.3, 0.5, -0.8, 0.05]):
        sets += list(D.plane_cut(blob, pl))
    assert max(m.nv for m in sets) > 2000
    rg, sg = g.hull_meshes(sets)
    ro, so = o.hull_meshes(sets)
    assert list(sg) == list(so)
    for i, (a, b) in enumerate(zip(rg, ro)):
        assert (a is None) == (b is None), i
        if a is not None:
            assert np.array_equal(a["tris"], b["tris"]) and a["volume"] == b["volume"], i


def test_hull_block_widths(tree_mod, oracle):
    """Large parts on every block width: on 152 SMs a batch of 320 parts
    runs on 256-thread blocks (8 picks per round), its first 200 parts on
    512-thread blocks (two per SM) and its first 8 on 1024-thread blocks (one
    per SM, 16 picks per round); all give the oracle's faces and volumes."""
    D = importlib.import_module("cuacd-web_gb300.decompose")
    cfg = dict(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=16384)
    g = tree_mod.GpuTree(**cfg)
    o = oracle.OracleTree(**cfg)
    blob = M.normalize(gen.blob_mesh(12, 44, seed=4))[0]
    sets = list(D.plane_cut(blob, [0.3, 0.5, -0.8, 0.05]))
    rng = np.random.default_rng(21)
    while len(sets) < 320:
        n = int(rng.integers(1100, 1500))
        s = rng.normal(size=(n, 3))
        s /= np.linalg.norm(s, axis=1, keepdims=True)
        s *= rng.uniform(0.8, 1.0, size=(n, 1))
        sets.append(M.Mesh(s.astype(np.float32), np.zeros((0, 3), np.uint32)))
    ro, so = o.hull_meshes(sets)
    for subset in (sets, sets[:200], sets[:8]):
        rg, sg = g.hull_meshes(subset)
        assert list(sg) == list(so[: len(subset)])
        for i, (a, b) in enumerate(zip(rg, ro)):
            assert (a is None) == (b is None), i
            if a is not None:
                assert np.array_equal(a["tris"], b["tris"]) and a["volume"] == b["volume"], i


def hd_pairs(oracle):
    t = oracle.OracleTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096)
    pairs = []
    for m in (M.l_shape(), square_torus(), stairs(), l_prism(), gen.staircase(8), gen.noisy_icosphere(3, seed=5)):
        h = t.hull_meshes([m])[0][0]
        pairs.append((m, M.Mesh(m.verts, h["tris"])))
    pairs.append((M.unit_cube(), M.make_box((0.1, 0, 0), (1.1, 1, 1))))
    return pairs


def test_hausdorff_matches_oracle_and_cpu(tree_mod, oracle):
    g = tree_mod.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0)
    pairs = hd_pairs(oracle)
    hg = g.hausdorff(pairs)
    ho = oracle.hausdorff_gpu_form(pairs)
    for i, (a, b) in enumerate(pairs):
        assert abs(hg[i] - ho[i]) <= 1e-5 + 1e-4 * ho[i], (i, hg[i], ho[i])
        c = oracle.hausdorff_cpu(a, b)
        assert abs(hg[i] - c) <= 1e-4 + 1e-3 * c, (i, hg[i], c)
    # known answers (tests/cpu.test.ts:78-87)
    assert 0.3 < hg[0] < 0.6
    assert abs(hg[-1] - 0.1) < 0.02


def test_hulls_with_hausdorff(tree_mod, oracle):
    g = tree_mod.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096)
    o = oracle.OracleTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096)
    meshes = [M.unit_cube(), M.l_shape(), square_torus(), stairs(), gen.staircase(8)]
    rg = g.hulls_with_hausdorff(meshes)
    ro, _ = o.hull_meshes(meshes)
    for m, a, b in zip(meshes, rg, ro):
        assert a is not None and b is not None
        assert np.array_equal(a["tris"], b["tris"]) and a["volume"] == b["volume"]
        ref = oracle.hausdorff_gpu_form([(m, M.Mesh(m.verts, b["tris"]))])[0]
        assert abs(a["hausdorff"] - ref) <= 1e-5 + 1e-4 * ref
    assert rg[0]["hausdorff"] < 1e-6


def test_hausdorff_screen_matches_exhaustive(tree_mod, oracle):
    """Target meshes of 256 triangles or more go through the tensor-core
    screen, which skips only triangles that cannot hold a sample's nearest
    point: its distances are the exhaustive search's bit for bit, on meshes
    against their hulls (samples on shared faces, distance 0 to many
    triangles) and on two different surfaces."""
    cfg = dict(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096)
    on = tree_mod.GpuTree(**cfg)
    off = tree_mod.GpuTree(**cfg, hdScreenMinTris=-1)
    pairs = []
    for seed, (nb, grid) in enumerate([(4, 20), (8, 28), (12, 36)]):
        m = gen.blob_mesh(nb, grid, seed=seed)
        h = on.hull_meshes([m])[0][0]
        pairs.append((m, M.Mesh(m.verts, h["tris"])))
    pairs.append((gen.noisy_icosphere(4, seed=1), gen.noisy_icosphere(4, seed=2)))
    pairs.append((gen.noisy_icosphere(3, seed=3), M.unit_cube()))
    a = on.hausdorff(pairs)
    st = on.hd_stats()
    b = off.hausdorff(pairs)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (a, b)
    assert st["screened"] > 0 and 0 < st["exact"] < st["screened"] and not st["timeout"], st
    assert off.hd_stats()["screened"] == 0
    # the fused hull + Hausdorff batch
    meshes = [p[0] for p in pairs[:3]]
    ra = on.hulls_with_hausdorff(meshes)
    rb = off.hulls_with_hausdorff(meshes)
    for x, y in zip(ra, rb):
        assert np.float32(x["hausdorff"]).view(np.uint32) == np.float32(y["hausdorff"]).view(np.uint32)
        assert np.array_equal(x["tris"], y["tris"])


def test_hausdorff_scratch_error(tree_mod):
    g = tree_mod.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, scratchWords=1000)
    with pytest.raises(tree_mod.ScratchError) as e:
        g.hausdorff([(M.unit_cube(), M.unit_cube())])
    assert "scratch" in str(e.value)


def test_empty_batches(tree_mod):
    g = tree_mod.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0)
    assert len(g.hausdorff([])) == 0
    assert g.hull_meshes([])[0] == []
    assert g.hulls_with_hausdorff([]) == []


def test_hull_batch_compact_readback_matches_single_batches(tree_mod):
    """A hull batch whose export range is large (one 10,242-point hull sets
    the stride of 80 meshes: about 20 MB) reads back each hull's own faces;
    faces, counts and volumes equal those of the same meshes hulled one per
    batch (whole-range readback)."""
    meshes = [gen.noisy_icosphere(5, seed=1)] + [gen.noisy_icosphere(2 + (k % 2), seed=k) for k in range(79)]
    g = tree_mod.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=16384, vertexCap=64 << 20,
                         triCap=64 << 20, scratchWords=64 << 20, hullBudgetBytes=1 << 30)
    many, st = g.hull_meshes(meshes)
    assert all(s == 0 for s in st)
    for m, h in zip(meshes, many):
        (one,), (s1,) = g.hull_meshes([m])
        assert s1 == 0 and one["volume"] == h["volume"] and np.array_equal(one["tris"], h["tris"])
