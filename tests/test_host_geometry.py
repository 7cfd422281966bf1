"""Host geometry of the decomposition loop (csrc/host_mesh.cpp,
csrc/plane_cut.cpp) against the oracle: the capped plane cut
(src/cpu/cut.ts) and the concave-edge planes (src/cpu/concave.ts). Runs on
the CPU; the library is only loaded, no GPU call is made.

Cut parity: the half meshes' vertex arrays are the oracle's (same positions
in the same order, up to a cap fan centroid on the plane that one clipper
adds where the other clips), their volumes agree to 1e-6
relative (the float32 cap vertices are not exactly coplanar, so two
triangulations of one cap differ in the last bits) and both are closed. Cap
triangles may differ: the reference
triangulates caps with earcut@3.0.1 (absent here) and both ear clippers are
this project's own, so only what the reference pins (closedness, volume,
n + 2h - 2) is compared."""
import zlib

import numpy as np
import pytest

from conftest import pkg
from fixtures import M, l_prism, square_torus, stairs

D = pkg("decompose")
G = pkg("meshgen")


def _meshes():
    out = [("cube", M.unit_cube()), ("l_shape", M.l_shape()), ("torus", square_torus()), ("stairs", stairs()),
           ("l_prism", l_prism()), ("staircase8", G.staircase(8)), ("ico3", G.noisy_icosphere(3, seed=1)),
           # marching-tetrahedra surface: vertices on shared grid lines and planes
           ("blob", M.normalize(G.blob_mesh(6, 26, seed=3))[0])]
    return out


def _planes(m, n, seed):
    rng = np.random.default_rng(seed)
    v = m.verts.astype(np.float64)
    lo, hi = v.min(0), v.max(0)
    out = [[1, 0, 0, -(lo[0] + hi[0]) / 2], [0, 1, 0, -(lo[1] + hi[1]) / 2], [0, 0, 1, -(lo[2] + hi[2]) / 2]]
    for _ in range(n):
        nrm = rng.normal(size=3)
        nrm /= np.linalg.norm(nrm)
        p = lo + rng.uniform(0.2, 0.8, 3) * (hi - lo)
        out.append([nrm[0], nrm[1], nrm[2], -float(nrm @ p)])
    return out


@pytest.mark.parametrize("name,mesh", _meshes())
def test_plane_cut_matches_oracle(oracle, name, mesh):
    for pl in _planes(mesh, 12, zlib.crc32(name.encode())):
        ref = oracle.plane_cut(mesh, pl)
        try:
            got = D.plane_cut(mesh, pl)
        except pkg("tree").CuacdError:
            got = None
        assert (ref is None) == (got is None), (name, pl)
        if ref is None:
            continue
        for r, g in zip(ref, got):
            rv = np.asarray(r.verts, np.float32).reshape(-1, 3)
            # the vertices before any cap fan centroid are the same; a cap
            # that one clipper triangulates and the other fans adds one
            # centroid on the cut plane at the end
            n = min(len(rv), len(g.verts))
            assert np.array_equal(rv[:n], g.verts[:n]), (name, pl)
            extra = np.concatenate([rv[n:], g.verts[n:]]).astype(np.float64)
            nrm = np.asarray(pl[:3], np.float64)
            assert np.all(np.abs(extra @ nrm + pl[3]) <= 1e-5 * np.linalg.norm(nrm)), (name, pl)
            assert M.is_closed(g), (name, pl)
            vr, vg = M.signed_volume(r), M.signed_volume(g)
            assert vg > 0
            assert abs(vr - vg) <= 1e-6 * abs(vr) + 1e-9, (name, pl, vr, vg)


def test_plane_cut_reference_cases():
    # tests/cpu.test.ts:18-56: halves of the cube, the L at its junction, the
    # torus through its hole
    pos, neg = D.plane_cut(M.unit_cube(), [1, 0, 0, -0.5])
    assert abs(M.volume(pos) - 0.5) < 1e-6 and abs(M.volume(neg) - 0.5) < 1e-6
    with pytest.raises(pkg("tree").CuacdError, match="does not split"):
        D.plane_cut(M.unit_cube(), [1, 0, 0, -1])
    pos, neg = D.plane_cut(M.l_shape(), [1, 0, 0, -1])
    assert M.is_closed(pos) and M.is_closed(neg)
    assert abs(M.volume(pos) - 0.5) < 1e-6 and abs(M.volume(neg) - 1) < 1e-6
    pos, neg = D.plane_cut(square_torus(), [0, 0, 1, 0])
    assert M.is_closed(pos) and M.is_closed(neg)
    assert abs(M.volume(pos) - 0.75) < 1e-6 and abs(M.volume(neg) - 0.75) < 1e-6
    # the cap is a ring (one hole): clipped with n + 2h - 2 triangles, so no
    # fan centroid joins the 8 top corners and 16 edge crossings
    assert pos.nv == 24 and pos.nt == 32 + 16


@pytest.mark.parametrize("name,mesh", _meshes())
def test_concave_planes_match_oracle(oracle, name, mesh):
    for seed in (12345, 7919, 3):
        for n in (1, 4, 16):
            ref = oracle.concave_planes(mesh, n, 0.005, 3.49, seed)
            got = D.concave_planes(mesh, n, 0.005, 3.49, seed)
            assert np.array_equal(np.asarray(ref, np.float32), got), (name, seed, n)


def test_concave_planes_reference_case():
    # tests/cpu.test.ts:89-95: the L prism's one concave edge gives 4 planes
    assert D.concave_planes(l_prism(), 8).shape == (4, 4)
    assert len(D.concave_planes(M.l_shape(), 8)) == 0
    assert len(D.concave_planes(M.unit_cube(), 8)) == 0


def _slab(mesh, axis, at, width):
    """The piece of mesh between two parallel planes `width` apart (the thin
    slabs a decomposition slices off a flat stretch of surface)."""
    n = [0.0, 0.0, 0.0]
    n[axis] = 1.0
    lo_pos, _ = D.plane_cut(mesh, n + [-at])  # x_axis >= at
    _, slab = D.plane_cut(lo_pos, n + [-(at + width)])  # and <= at + width
    return slab


def test_plane_cut_of_thin_slabs_matches_oracle(oracle):
    """Caps of thin slabs: long runs of nearly collinear boundary vertices
    (the cut crosses the earlier caps along straight lines), the degenerate
    polygons the ear clipper's flat mode handles."""
    checked = 0
    for mesh in (G.noisy_icosphere(3, seed=2), M.normalize(G.blob_mesh(6, 26, seed=3))[0], G.carved_sphere(3, 3, seed=2)):
        v = mesh.verts.astype(np.float64)
        lo, hi = v.min(0), v.max(0)
        for axis, frac, width in ((1, 0.45, 0.004), (0, 0.6, 0.002), (2, 0.3, 0.01)):
            try:
                slab = _slab(mesh, axis, lo[axis] + frac * (hi[axis] - lo[axis]), width * (hi[axis] - lo[axis]))
            except pkg("tree").CuacdError:
                continue
            sv = slab.verts.astype(np.float64)
            c = (sv.min(0) + sv.max(0)) / 2
            for pl in ([1, 0, 0, -c[0]], [0, 1, 0, -c[1]], [0, 0, 1, -c[2]], [0.6, 0.8, 0.0, -(0.6 * c[0] + 0.8 * c[1])]):
                ref = oracle.plane_cut(slab, pl)
                try:
                    got = D.plane_cut(slab, pl)
                except pkg("tree").CuacdError:
                    got = None
                assert (ref is None) == (got is None), (axis, pl)
                if ref is None:
                    continue
                for r, g in zip(ref, got):
                    rv = np.asarray(r.verts, np.float32).reshape(-1, 3)
                    k = min(len(rv), len(g.verts))
                    assert np.array_equal(rv[:k], g.verts[:k])
                    assert M.is_closed(g)
                    vr, vg = M.signed_volume(r), M.signed_volume(g)
                    assert abs(vr - vg) <= 1e-6 * abs(vr) + 1e-12, (vr, vg)
                checked += 1
    assert checked >= 12, checked
