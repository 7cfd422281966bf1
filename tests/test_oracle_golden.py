"""Pins the CPU oracle against the reference's own known answers
(tests/cpu.test.ts, tests/gpu_tree.test.ts) and the reference's quickhull."""
import numpy as np
import pytest

import tree_cases
from fixtures import M, l_prism, square_torus, stairs


def test_fixtures_closed_outward():
    for m in (M.unit_cube(), M.l_shape(), square_torus(), stairs(), l_prism()):
        assert M.is_closed(m)
        assert M.signed_volume(m) > 0
    assert abs(M.volume(square_torus()) - 1.5) < 1e-6
    assert abs(M.volume(M.l_shape()) - 1.5) < 1e-6


def test_plane_cut_cube(oracle):
    cube = M.unit_cube()
    for pl in ([1, 0, 0, -0.5], [0, 1, 0, -0.3], [0, 0, 1, -0.75], [0.6, 0.8, 0, -0.7]):
        pos, neg = oracle.plane_cut(cube, pl)
        assert M.is_closed(pos) and M.is_closed(neg)
        assert M.signed_volume(pos) > 0 and M.signed_volume(neg) > 0
        assert abs(M.volume(pos) + M.volume(neg) - 1) < 1e-6
    pos, _ = oracle.plane_cut(cube, [1, 0, 0, -0.5])
    assert abs(M.volume(pos) - 0.5) < 1e-6


def test_plane_cut_on_plane(oracle):
    assert oracle.plane_cut(M.unit_cube(), [1, 0, 0, -1]) is None
    pos, neg = oracle.plane_cut(M.l_shape(), [1, 0, 0, -1])
    assert M.is_closed(pos) and M.is_closed(neg)
    assert abs(M.volume(pos) - 0.5) < 1e-6 and abs(M.volume(neg) - 1) < 1e-6


def test_plane_cut_torus_holes(oracle):
    t = square_torus()
    pos, neg = oracle.plane_cut(t, [0, 0, 1, 0])
    assert M.is_closed(pos) and M.is_closed(neg)
    assert abs(M.volume(pos) - 0.75) < 1e-6 and abs(M.volume(neg) - 0.75) < 1e-6
    pos, neg = oracle.plane_cut(t, [1, 0, 0, 0])
    assert M.is_closed(pos) and M.is_closed(neg)
    assert abs(M.volume(pos) + M.volume(neg) - 1.5) < 1e-6


@pytest.mark.parametrize("use_ref", [True, False])
def test_hull_volumes(oracle, use_ref):
    if use_ref and not oracle.qh_ref_loaded():
        pytest.skip("reference quickhull not built here")
    assert abs(oracle.hull_volume(M.unit_cube(), use_ref) - 1) < 1e-6
    assert abs(oracle.hull_volume(M.l_shape(), use_ref) - 1.75) < 1e-6
    s = 1
    pts = []
    for _ in range(3000):
        s = (s * 16807) % 2147483647
        pts.append(s / 2147483647 * 2 - 1)
    v = oracle.hull_volume(M.Mesh(np.array(pts, np.float32), np.zeros((0, 3), np.uint32)), use_ref)
    assert 6.5 < v < 8


def test_oracle_hull_matches_reference_quickhull(oracle):
    """The oracle's grid hull against the reference's quickhull on random
    clouds and noisy spheres: relative volume error within the 2^21 grid's
    quantisation (the reference measured 2.3e-5 worst against qhull)."""
    if not oracle.qh_ref_loaded():
        pytest.skip("reference quickhull not built here")
    mg = __import__("fixtures").M  # noqa
    import importlib

    gen = importlib.import_module("cuacd-web_gb300.meshgen")
    rng = np.random.default_rng(0)
    clouds = [rng.normal(size=(n, 3)).astype(np.float32) for n in (10, 50, 300, 2000)]
    clouds.append(gen.noisy_icosphere(3).verts)
    for c in clouds:
        m = M.Mesh(c, np.zeros((0, 3), np.uint32))
        a, b = oracle.hull_volume(m, True), oracle.hull_volume(m, False)
        assert abs(a - b) <= 3e-5 * a, (len(c), a, b)


def test_oracle_hull_faces_closed(oracle):
    import importlib

    gen = importlib.import_module("cuacd-web_gb300.meshgen")
    t = oracle.OracleTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096)
    m = gen.noisy_icosphere(3)
    res, status = t.hull_meshes([m, M.unit_cube(), M.l_shape()])
    for r, src in zip(res, (m, M.unit_cube(), M.l_shape())):
        assert r is not None
        h = M.Mesh(src.verts, r["tris"])
        assert M.is_closed(h)
        assert M.signed_volume(h) > 0
        assert abs(M.volume(h) - r["volume"]) < 1e-4 * r["volume"]


def test_hausdorff_cpu_known_answers(oracle):
    cube = M.unit_cube()
    t = oracle.OracleTree(width=3, width2=3, depth=1, nConcaveEdges=0)
    hull = t.hull_meshes([cube])[0][0]
    assert oracle.hausdorff_cpu(cube, M.Mesh(cube.verts, hull["tris"])) < 1e-6
    L = M.l_shape()
    hl = t.hull_meshes([L])[0][0]
    hd = oracle.hausdorff_cpu(L, M.Mesh(L.verts, hl["tris"]))
    assert 0.3 < hd < 0.6, hd
    a, b = M.make_box((0, 0, 0), (1, 1, 1)), M.make_box((0.1, 0, 0), (1.1, 1, 1))
    assert abs(oracle.hausdorff_cpu(a, b) - 0.1) < 0.02


def test_hausdorff_gpu_form_matches_cpu(oracle):
    """cpu.test.ts:97-111: the GPU form within 1e-4 + 1e-3 * cpu."""
    t = oracle.OracleTree(width=3, width2=3, depth=1, nConcaveEdges=0)
    pairs = []
    for m in (M.l_shape(), square_torus(), stairs()):
        h = t.hull_meshes([m])[0][0]
        pairs.append((m, M.Mesh(m.verts, h["tris"])))
    pairs.append((M.unit_cube(), M.make_box((0.1, 0, 0), (1.1, 1, 1))))
    g = oracle.hausdorff_gpu_form(pairs)
    for (a, b), gv in zip(pairs, g):
        c = oracle.hausdorff_cpu(a, b)
        assert abs(gv - c) <= 1e-4 + 1e-3 * c, (gv, c)


def test_concave_planes(oracle):
    assert oracle.concave_planes(l_prism(), 8).shape == (4, 4)
    assert len(oracle.concave_planes(M.l_shape(), 8)) == 0
    assert len(oracle.concave_planes(M.unit_cube(), 8)) == 0


@pytest.mark.parametrize("case", tree_cases.ALL, ids=lambda c: c.__name__)
def test_oracle_tree_known_answers(oracle, case):
    case(oracle.OracleTree)
