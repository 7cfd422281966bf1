"""The capped plane cut on the GPU (cuacd_tree_plane_cuts, csrc/cut_kernels.cu)
against the host cut (cuacd_plane_cut, csrc/plane_cut.cpp) and the oracle's
restatement of src/cpu/cut.ts.

GPU against host: bit for bit — every half's vertex array (positions and
order) and triangle array, and every failure (a plane that does not split
the mesh fails both). GPU against the oracle: the halves' vertices are the
oracle's (same positions in the same order, up to a cap fan centroid on the
cut plane that one ear clipper adds where the other clips), volumes agree to
1e-6 relative, both halves are closed. Cap triangles are not compared with
the oracle: the reference triangulates caps with earcut@3.0.1, absent here,
so exact cap triangles are unpinned (closedness, volume and the n + 2h - 2
count are what the reference pins).
"""
import zlib

import numpy as np
import pytest

from conftest import pkg
from fixtures import M, l_prism, square_torus, stairs

pytestmark = pytest.mark.gpu

D = pkg("decompose")
G = pkg("meshgen")
T = pkg("tree")


def _tree():
    return T.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0)


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


def _meshes():
    return [("cube", M.unit_cube()), ("l_shape", M.l_shape()), ("torus", square_torus()), ("stairs", stairs()),
            ("l_prism", l_prism()), ("staircase8", G.staircase(8)),
            ("staircase8_188", G.staircase(8, wall_centroids=True)), ("ico3", G.noisy_icosphere(3, seed=1)),
            ("ico4", G.noisy_icosphere(4, seed=0)),
            # marching-tetrahedra surfaces: vertices on shared grid lines and planes
            ("blob", M.normalize(G.blob_mesh(6, 26, seed=3))[0]),
            ("blob_big", M.normalize(G.blob_mesh(12, 48, seed=5))[0]),
            ("carved", G.carved_sphere(3, 3, seed=2))]


def _host_cut(mesh, pl):
    try:
        return D.plane_cut(mesh, pl)
    except T.CuacdError:
        return None


def _same(a, b):
    return (np.array_equal(a.verts.view(np.uint32), b.verts.view(np.uint32)) and a.tris.shape == b.tris.shape
            and np.array_equal(a.tris, b.tris))


def test_gpu_cut_matches_host_cut_bit_for_bit():
    g = _tree()
    meshes = _meshes()
    planes, idx, names = [], [], []
    for k, (name, m) in enumerate(meshes):
        for pl in _planes(m, 10, zlib.crc32(name.encode())):
            planes.append(pl)
            idx.append(k)
            names.append(name)
        # a plane through vertices (on-plane vertices on both halves), and
        # planes beside the mesh (no split)
        v = m.verts.astype(np.float64)
        planes += [[0, 0, 1, -float(v[0, 2])], [1, 0, 0, -float(v[:, 0].max()) - 1.0],
                   [0, 1, 0, -float(v[:, 1].min())]]
        idx += [k, k, k]
        names += [name] * 3
    got = g.plane_cuts([m for _, m in meshes], planes, idx)
    n_ok = n_fail = 0
    for (st, pos, neg), pl, k, name in zip(got, planes, idx, names):
        ref = _host_cut(meshes[k][1], pl)
        assert (ref is None) == (st != 0), (name, pl, st)
        if ref is None:
            n_fail += 1
            continue
        n_ok += 1
        assert _same(pos, ref[0]) and _same(neg, ref[1]), (name, pl)
    assert n_ok > 100 and n_fail >= len(meshes)


def test_gpu_cut_config1_icosphere_96_planes(oracle):
    # the icosphere configuration: level 4 (2,562 vertices, 5,120 triangles),
    # radial noise, 96 seeded planes, one batch
    m = G.noisy_icosphere(4, noise=0.15, seed=0)
    planes = G.random_planes(m, 96, seed=0).astype(np.float64)
    got = _tree().plane_cuts([m], planes, np.zeros(96, np.int32))
    for (st, pos, neg), pl in zip(got, planes):
        ref = _host_cut(m, pl)
        assert (ref is None) == (st != 0)
        if ref is None:
            continue
        assert _same(pos, ref[0]) and _same(neg, ref[1])
        orc = oracle.plane_cut(m, pl)
        for r, h in zip(orc, (pos, neg)):
            rv = np.asarray(r.verts, np.float32).reshape(-1, 3)
            n = min(len(rv), len(h.verts))
            assert np.array_equal(rv[:n], h.verts[:n])
            assert M.is_closed(h)
            vr, vg = M.signed_volume(r), M.signed_volume(h)
            assert abs(vr - vg) <= 1e-6 * abs(vr) + 1e-9


@pytest.mark.parametrize("name,mesh", _meshes())
def test_gpu_cut_matches_oracle(oracle, name, mesh):
    planes = _planes(mesh, 8, zlib.crc32(name.encode()) + 1)
    got = _tree().plane_cuts([mesh], planes, np.zeros(len(planes), np.int32))
    for (st, pos, neg), pl in zip(got, planes):
        ref = oracle.plane_cut(mesh, pl)
        assert (ref is None) == (st != 0), (name, pl)
        if ref is None:
            continue
        for r, h in zip(ref, (pos, neg)):
            rv = np.asarray(r.verts, np.float32).reshape(-1, 3)
            n = min(len(rv), len(h.verts))
            assert np.array_equal(rv[:n], h.verts[:n]), (name, pl)
            extra = np.concatenate([rv[n:], h.verts[n:]]).astype(np.float64)
            nrm = np.asarray(pl[:3], np.float64)
            assert np.all(np.abs(extra @ nrm + pl[3]) <= 1e-5 * np.linalg.norm(nrm)), (name, pl)
            assert M.is_closed(h), (name, pl)
            vr, vg = M.signed_volume(r), M.signed_volume(h)
            assert abs(vr - vg) <= 1e-6 * abs(vr) + 1e-9, (name, pl, vr, vg)


def test_gpu_cut_reference_cases():
    # tests/cpu.test.ts:18-56 through the GPU cut: cube halves, the L at its
    # junction, the torus through its hole (an annulus cap: one hole)
    g = _tree()
    cube, ell, tor = M.unit_cube(), M.l_shape(), square_torus()
    got = g.plane_cuts([cube, ell, tor], [[1, 0, 0, -0.5], [1, 0, 0, -1], [1, 0, 0, -1], [0, 0, 1, 0]], [0, 0, 1, 2])
    (s0, p0, n0), (s1, _, _), (s2, p2, n2), (s3, p3, n3) = got
    assert s0 == 0 and abs(M.volume(p0) - 0.5) < 1e-6 and abs(M.volume(n0) - 0.5) < 1e-6
    assert s1 == 1  # the plane does not split the cube
    assert s2 == 0 and abs(M.volume(p2) - 0.5) < 1e-6 and abs(M.volume(n2) - 1) < 1e-6
    assert s3 == 0 and M.is_closed(p3) and M.is_closed(n3)
    assert abs(M.volume(p3) - 0.75) < 1e-6 and p3.nv == 24 and p3.nt == 32 + 16


def test_eval_cuts_matches_cpu_helpers(oracle):
    """The icosphere configuration through cuacd_tree_eval_cuts (GPU cut, hull
    and Hausdorff of every half) against the oracle's restatement of the
    reference's CPU helpers (planeCut, grid hull, volumes, rv and the BVH
    Hausdorff of src/cpu/hausdorff.ts in double): the same planes split,
    volumes within 1e-6, hull volumes within 1e-5 relative, rv within 1e-5
    and Hausdorff within the reference's own 1e-4 + 1e-3 d (cpu.test.ts:97-111)."""
    m = G.noisy_icosphere(4, noise=0.15, seed=0)
    planes = G.random_planes(m, 24, seed=0).astype(np.float64)
    g = T.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096, scratchWords=64 << 20)
    got = g.eval_cuts(m, planes)
    ref = oracle.eval_candidates(m, planes, threads=4, with_hd=True, use_ref=False)
    assert np.array_equal(got[:, 0], ref[:, 0]) and got[:, 0].sum() > 12
    ok = got[:, 0] == 1
    assert np.allclose(got[ok, 1:3], ref[ok, 1:3], rtol=1e-6, atol=1e-9)
    assert np.allclose(got[ok, 3:5], ref[ok, 3:5], rtol=1e-5, atol=1e-7)
    assert np.allclose(got[ok, 5:7], ref[ok, 5:7], rtol=0, atol=1e-5)
    d = ref[ok, 7]
    assert np.all(np.abs(got[ok, 7] - d) <= 1e-4 + 1e-3 * d), np.abs(got[ok, 7] - d).max()


def _open_meshes():
    cube = M.unit_cube()
    ico = G.noisy_icosphere(3, seed=2)
    blob = M.normalize(G.blob_mesh(6, 26, seed=3))[0]
    return [("cube_open", M.Mesh(cube.verts, cube.tris[2:])),
            ("ico_cap_removed", M.Mesh(ico.verts, ico.tris[ico.verts[ico.tris][:, :, 2].mean(1) < 0.8])),
            ("blob_half_shell", M.Mesh(blob.verts, blob.tris[blob.verts[blob.tris][:, :, 0].mean(1) < 0.1])),
            ("strip", M.Mesh(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0.2], [0, 2, 0], [1, 2, 0.4]], np.float32),
                             np.array([[0, 1, 2], [1, 3, 2], [2, 3, 4], [3, 5, 4]], np.uint32)))]


def test_gpu_cut_open_meshes_match_host_cut():
    # open meshes: boundary edges off the plane (the open rims) join the
    # boundary loops, so most of these cuts fail as the host cut's do, with
    # the same reason
    g = _tree()
    meshes = _open_meshes()
    planes, idx = [], []
    for k, (name, m) in enumerate(meshes):
        for pl in _planes(m, 6, zlib.crc32(name.encode())):
            planes.append(pl)
            idx.append(k)
    got = g.plane_cuts([m for _, m in meshes], planes, idx)
    for (st, pos, neg), pl, k in zip(got, planes, idx):
        name, m = meshes[k]
        try:
            ref = D.plane_cut(m, pl)
            err = None
        except T.CuacdError as x:
            ref, err = None, str(x)
        assert (ref is None) == (st != 0), (name, pl, st, err)
        if ref is None:
            reason = {1: "does not split", 2: "open boundary chain", 3: "dead end", 4: "cycle"}.get(st)
            assert reason is not None and reason in err, (name, st, err)
            continue
        assert _same(pos, ref[0]) and _same(neg, ref[1]), (name, pl)


def test_gpu_cut_closed_flag_gives_the_same_halves():
    g = _tree()
    meshes = [m for _, m in _meshes()]
    planes, idx = [], []
    for k, m in enumerate(meshes):
        for pl in _planes(m, 3, 99 + k):
            planes.append(pl)
            idx.append(k)
    a = g.plane_cuts(meshes, planes, idx, closed=False)
    b = g.plane_cuts(meshes, planes, idx, closed=True)
    for x, y in zip(a, b):
        assert x[0] == y[0]
        if x[0] == 0:
            assert _same(x[1], y[1]) and _same(x[2], y[2])


def test_device_halves_feed_the_next_calls():
    """cuacd_cuts_half_device: the halves of a GPU cut batch, passed as device
    meshes to the next hull batch, concave-plane batch, tree run and cut
    batch (the decomposer's resident parts), give the results of the same
    halves passed from host memory. The last cut reads its inputs from the
    output buffers it then overwrites."""
    import ctypes as C

    A = pkg("_abi")
    L = T.load_library()
    L.cuacd_cuts_half_device.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.POINTER(C.c_float)),
                                         C.POINTER(C.POINTER(C.c_uint32))]
    m = G.noisy_icosphere(3, seed=1)
    g = T.GpuTree(width=6, width2=3, depth=2, nConcaveEdges=16, hullMaxVerts=4096)
    c = (m.verts.min(0).astype(np.float64) + m.verts.max(0)) / 2
    planes = np.ascontiguousarray([[1.0, 0.0, 0.0, -c[0] - 0.05], [0.0, 1.0, 0.0, -c[1] + 0.1]], np.float64)
    ma = A.MeshArray([m])
    idx = np.zeros(2, np.int32)
    h = C.c_void_p()
    assert L.cuacd_tree_plane_cuts(g.h, ma.arr, 1, idx.ctypes.data_as(C.POINTER(C.c_int32)),
                                   planes.ctypes.data_as(C.POINTER(C.c_double)), 2, 1, C.byref(h)) == 0
    host, dev = [], (A.MeshRef * 4)()
    for k in range(2):
        for sd in range(2):
            v, t = C.POINTER(C.c_float)(), C.POINTER(C.c_uint32)()
            nv, nt = C.c_uint32(), C.c_uint32()
            assert L.cuacd_cuts_half(h, k, sd, C.byref(v), C.byref(nv), C.byref(t), C.byref(nt)) == 0
            host.append(M.Mesh(np.ctypeslib.as_array(v, shape=(3 * nv.value,)).reshape(-1, 3).copy(),
                               np.ctypeslib.as_array(t, shape=(3 * nt.value,)).reshape(-1, 3).copy()))
            dv, dt = C.POINTER(C.c_float)(), C.POINTER(C.c_uint32)()
            assert L.cuacd_cuts_half_device(h, k, sd, C.byref(dv), C.byref(dt)) == 0
            i = 2 * k + sd
            dev[i].verts, dev[i].tris, dev[i].nv, dev[i].nt = dv, dt, nv.value, nt.value
    L.cuacd_cuts_free(h)
    n = 4
    # hulls
    hh, _ = g.hull_meshes(host)
    stride = 3 * 2 * max(x.nv for x in host)
    tris = np.zeros(n * stride, np.uint32)
    vol = np.zeros(n, np.float32)
    ntr = np.zeros(n, np.uint32)
    st = np.zeros(n, np.int32)
    assert L.cuacd_tree_hull_meshes(g.h, dev, n, 0, A.uptr(tris), stride, A.fptr(vol), A.uptr(ntr),
                                    st.ctypes.data_as(C.POINTER(C.c_int32))) == 0
    for k in range(n):
        assert st[k] == 0 and vol[k] == hh[k]["volume"]
        assert np.array_equal(tris[k * stride: k * stride + 3 * ntr[k]].reshape(-1, 3), hh[k]["tris"])
    # concave planes
    ph = g.concave_planes(host, 16)
    out = np.zeros((n, 64, 4), np.float32)
    cnt = np.zeros(n, np.int32)
    seeds = np.full(n, 12345, np.uint32)
    assert L.cuacd_tree_concave_planes(g.h, dev, n, 16, 0.005, 3.49, A.uptr(seeds), A.fptr(out),
                                       cnt.ctypes.data_as(C.POINTER(C.c_int32))) == 0
    for k in range(n):
        assert np.array_equal(out[k, : cnt[k]], ph[k])
    # tree run
    rh = g.run(host, ph)
    ep = np.zeros((n, g.plane_slots, 4), np.float32)
    for k in range(n):
        ep[k, : len(ph[k])] = ph[k]
    res = (A.SeedResult * n)()
    rs = A.RunStats()
    opts = A.RunOpts(depth=0, width=-1, nEdgeCuts=-1)
    assert L.cuacd_tree_run(g.h, dev, n, A.fptr(ep), g.plane_slots, C.byref(opts), res, C.byref(rs)) == 0
    rd = T._result(res, rs, n)
    assert rd["seeds"] == rh["seeds"] and rd["validJobs"] == rh["validJobs"]
    # a cut of the device halves, which overwrites the buffers they live in
    cp = np.ascontiguousarray([[0.0, 0.0, 1.0, -c[2] - 0.02]] * n, np.float64)
    ref = g.plane_cuts(host, cp, np.arange(n, dtype=np.int32), closed=True)
    # the host-mesh cut above replaced the batch the device halves lived in:
    # cut once more from host so that the device halves are fresh, then cut them
    h2 = C.c_void_p()
    assert L.cuacd_tree_plane_cuts(g.h, ma.arr, 1, idx.ctypes.data_as(C.POINTER(C.c_int32)),
                                   planes.ctypes.data_as(C.POINTER(C.c_double)), 2, 1, C.byref(h2)) == 0
    for k in range(2):
        for sd in range(2):
            dv, dt = C.POINTER(C.c_float)(), C.POINTER(C.c_uint32)()
            assert L.cuacd_cuts_half_device(h2, k, sd, C.byref(dv), C.byref(dt)) == 0
            dev[2 * k + sd].verts, dev[2 * k + sd].tris = dv, dt
    L.cuacd_cuts_free(h2)
    h3 = C.c_void_p()
    cidx = np.arange(n, dtype=np.int32)
    assert L.cuacd_tree_plane_cuts(g.h, dev, n, cidx.ctypes.data_as(C.POINTER(C.c_int32)),
                                   cp.ctypes.data_as(C.POINTER(C.c_double)), n, 1, C.byref(h3)) == 0
    for k in range(n):
        st_ref, pos, neg = ref[k]
        for sd, want in enumerate((pos, neg)):
            v, t = C.POINTER(C.c_float)(), C.POINTER(C.c_uint32)()
            nv, nt = C.c_uint32(), C.c_uint32()
            s = L.cuacd_cuts_half(h3, k, sd, C.byref(v), C.byref(nv), C.byref(t), C.byref(nt))
            assert (s == 0) == (st_ref == 0)
            if s == 0:
                got = M.Mesh(np.ctypeslib.as_array(v, shape=(3 * nv.value,)).reshape(-1, 3).copy(),
                             np.ctypeslib.as_array(t, shape=(3 * nt.value,)).reshape(-1, 3).copy())
                assert _same(got, want)
    L.cuacd_cuts_free(h3)
