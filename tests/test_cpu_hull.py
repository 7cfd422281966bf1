"""The reference's CPU hull and the output-hull cleanup on the host
(csrc/cpu_hull.cpp): quickhull (wasm/quickhull via wasm/qh.cpp) and
cleanHullFaces (src/cpu/hull.ts:87-155). Runs on the CPU; the library is
only loaded.

Parity: quickhull's vertex and triangle arrays are bit-identical to the
reference's own quickhull compiled from its sources (oracle/_ref, built
where the reference tree is present), on random, coplanar, collinear,
duplicated and grid point sets; cleanHullFaces' triangles are identical to
a Python restatement of hull.ts:87-155 running on that reference quickhull
(the one tolerance: Math.hypot, which no C library reproduces bit for bit,
only decides comparisons against thresholds)."""
import numpy as np
import pytest

from conftest import pkg
from fixtures import M, stairs

D = pkg("decompose")
G = pkg("meshgen")
Mesh = pkg("mesh").Mesh


def _need_ref(oracle):
    if oracle.qh_ref() is None:
        pytest.skip("oracle/_ref (the reference's quickhull) is built only where the reference tree is present")


def _point_sets():
    rng = np.random.default_rng(7)
    sets = [("cube", rng.uniform(-1, 1, (200, 3))),
            ("sphere", (lambda p: p / np.linalg.norm(p, axis=1, keepdims=True))(rng.normal(size=(300, 3)))),
            ("gauss", rng.normal(size=(500, 3)) * [1, 2, 0.5]),
            ("grid", np.stack(np.meshgrid(*[np.arange(5.0)] * 3), -1).reshape(-1, 3)),
            ("plane", np.c_[rng.uniform(-1, 1, (60, 2)), np.zeros(60)]),
            ("line", np.outer(np.linspace(0, 1, 20), [1, 2, 3])),
            ("dups", np.repeat(rng.uniform(-1, 1, (30, 3)), 3, axis=0)),
            ("one", np.tile([[0.5, 0.5, 0.5]], (8, 1)))]
    for n in (1, 2, 3, 4, 5):
        sets.append((f"n{n}", rng.uniform(-1, 1, (n, 3))))
    # cut halves: a planar cap of many coplanar points on a curved surface
    blob = pkg("mesh").normalize(G.blob_mesh(6, 24, 3))[0]
    for k, pl in enumerate([[1, 0, 0, 0.1], [0.3, 0.5, -0.8, 0.05]]):
        pos, neg = D.plane_cut(blob, pl)
        sets.append((f"half{k}", pos.verts.astype(np.float64)))
    for name, m in (("staircase8", G.staircase(8)), ("stairs", stairs()), ("ico3", G.noisy_icosphere(3, seed=1))):
        sets.append((name, m.verts.astype(np.float64)))
    return sets


@pytest.mark.parametrize("name,pts", _point_sets(), ids=[s[0] for s in _point_sets()])
@pytest.mark.parametrize("eps", [1e-7, 2e-5])
def test_quickhull_matches_reference(oracle, name, pts, eps):
    _need_ref(oracle)
    v, t = D.quickhull(pts, eps)
    rv, rt = oracle.quickhull_ref(pts, eps)
    assert np.array_equal(v, rv), name
    assert np.array_equal(t, rt), name


def test_quickhull_volume(oracle):
    # unit cube corners + interior points: volume 1, 12 triangles, 8 vertices
    rng = np.random.default_rng(1)
    pts = np.vstack([M.unit_cube().verts, rng.uniform(0.1, 0.9, (50, 3))]).astype(np.float64)
    v, t = D.quickhull(pts)
    assert v.shape == (8, 3) and t.shape == (12, 3)
    m = Mesh(v.astype(np.float32), t)
    assert abs(oracle.hull_volume(m, False) - 1.0) < 1e-9


def _raw_hull(pts32):
    """A closed hull of pts32 over its own indices with extra near-coplanar
    vertices (the kind of face set the exact grid hull exports)."""
    v, t = D.quickhull(pts32.astype(np.float64), 1e-13)
    key = {tuple(p): i for i, p in enumerate(pts32.astype(np.float64))}
    return np.array([[key[tuple(v[i])] for i in tri] for tri in t], np.uint32)


def _hull_inputs():
    rng = np.random.default_rng(3)
    out = []
    blob = pkg("mesh").normalize(G.blob_mesh(6, 24, 3))[0]
    for k, pl in enumerate([[1, 0, 0, 0.1], [0, 0, 1, -0.2], [0.3, 0.5, -0.8, 0.05]]):
        pos, neg = D.plane_cut(blob, pl)
        out.append((f"blobhalf{k}", pos.verts))
        out.append((f"blobhalf{k}n", neg.verts))
    out.append(("staircase8", G.staircase(8).verts))
    out.append(("stairs", stairs().verts))
    # points on a box's faces and edges: coplanar and collinear hull points
    f = rng.uniform(0, 1, (120, 3)).astype(np.float32)
    ax = rng.integers(0, 3, 120)
    f[np.arange(120), ax] = rng.integers(0, 2, 120).astype(np.float32)
    out.append(("boxfaces", np.vstack([M.unit_cube().verts, f])))
    return out


@pytest.mark.parametrize("name,pts", _hull_inputs(), ids=[s[0] for s in _hull_inputs()])
@pytest.mark.parametrize("eps", [2e-5, 1e-3])
def test_clean_hull_faces_matches_restatement(oracle, name, pts, eps):
    _need_ref(oracle)
    pts = np.asarray(pts, np.float32)
    raw = _raw_hull(pts)
    got = D.clean_hull_faces(pts, raw, eps)
    want = oracle.clean_hull_faces_ref(pts, raw, eps)
    assert np.array_equal(got, want), name


def _issues(V, T, P):
    # hull_output.test.ts:13-38: closed, outward, no degenerate faces,
    # every point inside within 1e-4 of the extent
    V = V.astype(np.float64)
    if not D_closed(T, len(V)):
        return "not closed"
    lo, hi = P.min(), P.max()
    ext = hi - lo
    bad = 0
    max_out = 0.0
    for a, b, c in T:
        u, w = V[b] - V[a], V[c] - V[a]
        n = np.cross(u, w)
        l = np.linalg.norm(n)
        if not l > 1e-6 * np.linalg.norm(u) * np.linalg.norm(w):
            bad += 1
            continue
        n /= l
        max_out = max(max_out, float((P.astype(np.float64) @ n - n @ V[a]).max()))
    if bad:
        return f"{bad} degenerate faces"
    if max_out > 1e-4 * ext:
        return f"points outside by {max_out / ext:.2e}"
    return None


def D_closed(T, nv):
    cnt = {}
    for t in T:
        for e in range(3):
            k = (int(t[e]), int(t[(e + 1) % 3]))
            cnt[k] = cnt.get(k, 0) + 1
    return all(c == 1 and cnt.get((b, a)) == 1 for (a, b), c in cnt.items())


@pytest.mark.parametrize("name,pts", _hull_inputs(), ids=[s[0] for s in _hull_inputs()])
def test_clean_hull_faces_output_quality(name, pts):
    # with the decomposer's epsilon the cleaned hull of a part has no
    # degenerate face and contains the part (hull_output.test.ts:13-38)
    pts = np.asarray(pts, np.float32)
    raw = _raw_hull(pts)
    got = D.clean_hull_faces(pts, raw, 2e-5)
    assert _issues(pts, got, pts) is None, name
    # the rebuilt faces keep the hull volume
    def vol(T):
        V = pts.astype(np.float64)
        a, b, c = V[T[:, 0]], V[T[:, 1]], V[T[:, 2]]
        return abs(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6)
    assert abs(vol(got) - vol(raw)) <= 10 * 2e-5 * vol(raw) + 1e-12


def test_clean_hull_faces_rejects_and_small():
    cube = M.unit_cube()
    # fewer than 4 triangles: returned as given
    t = cube.tris[:3]
    assert np.array_equal(D.clean_hull_faces(cube.verts, t), t)
    # a face set missing a face away from vertex 0 (the volume's anchor) has
    # another volume than its rebuilt hull: returned as given
    open_t = np.array([t for t in cube.tris if 0 not in t][1:] + [t for t in cube.tris if 0 in t], np.uint32)
    assert np.array_equal(D.clean_hull_faces(cube.verts, open_t), open_t)
    # a clean hull stays a closed 12-triangle hull of the same corners
    got = D.clean_hull_faces(cube.verts, cube.tris)
    assert got.shape == (12, 3) and D_closed(got, 8) and set(got.reshape(-1)) == set(range(8))


def test_quickhull_and_cleanup_edges():
    # no points, one point: no triangles and no error
    v, t = D.quickhull(np.zeros((0, 3)))
    assert v.shape == (0, 3) and t.shape == (0, 3)
    v, t = D.quickhull(np.array([[1.0, 2.0, 3.0]]))
    assert t.shape[0] == 4  # the reference's degenerate tetrahedron of repeated indices
    # an out-of-range triangle index is an error, not a read past the array
    cube = M.unit_cube()
    with pytest.raises(Exception):
        D.clean_hull_faces(cube.verts, np.array([[0, 1, 99]], np.uint32))
    # no triangles: nothing to clean
    assert D.clean_hull_faces(cube.verts, np.zeros((0, 3), np.uint32)).shape == (0, 3)
