"""The allocation-free hull entry point, through the C ABI.

cuacd_hull_points_noalloc serves callers that cannot allocate device memory
when they need a hull (their own arena or caching allocator owns the GPU, or
allocating would stall work already running). They pass device buffers they
own; the kernel's scratch is a fixed array inside the library. This test
allocates those caller buffers itself (with torch), calls the entry point
twice in a row on different point sets, and checks each result against the
allocating entry point cuacd_tree_hull_meshes: identical faces, volumes
within the tests' tolerance. It also checks that point sets beyond the
array's 4096-point limit and triangle buffers smaller than a hull of the
points may need are refused, and that fewer than 4 points give status 8.
The file is collected last so that a run stopping at the first failure has
run every other test first.
"""
import ctypes as C
import importlib

import numpy as np
import pytest

import parity

pytestmark = pytest.mark.gpu


def test_no_alloc_hull_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    tree = importlib.import_module("cuacd-web_gb300.tree")
    gen = importlib.import_module("cuacd-web_gb300.meshgen")
    lib = tree.load_library()
    fn = lib.cuacd_hull_points_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    g = tree.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096)
    # consecutive calls: 642 points and 50 points (warp groups), then 2562
    # points (a block group)
    for m in (gen.noisy_icosphere(3, seed=4), gen.staircase(8), gen.noisy_icosphere(4, seed=6)):
        ref, status_ref = g.hull_meshes([m])
        assert status_ref[0] == 0
        pts = torch.from_numpy(np.ascontiguousarray(m.verts)).cuda()
        cap = 6 * m.nv
        tris = torch.zeros(cap, dtype=torch.int32, device="cuda")
        vol = torch.zeros(1, dtype=torch.float32, device="cuda")
        nt = torch.zeros(1, dtype=torch.int32, device="cuda")
        st = torch.full((1,), -7, dtype=torch.int32, device="cuda")
        rc = fn(pts.data_ptr(), m.nv, tris.data_ptr(), cap, vol.data_ptr(), nt.data_ptr(), st.data_ptr(), None)
        assert rc == 0, lib.cuacd_last_error().decode()
        torch.cuda.synchronize()
        assert st.item() == 0
        n = nt.item()
        got = tris[: 3 * n].cpu().numpy().astype(np.uint32).reshape(-1, 3)
        assert np.array_equal(got, ref[0]["tris"])
        assert parity.close([vol.item()], [ref[0]["volume"]])


def test_no_alloc_rejects_point_sets_beyond_the_limit():
    torch = pytest.importorskip("torch")
    tree = importlib.import_module("cuacd-web_gb300.tree")
    lib = tree.load_library()
    fn = lib.cuacd_hull_points_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    pts = torch.zeros(3 * 5000, dtype=torch.float32, device="cuda")
    out = torch.zeros(64, dtype=torch.int32, device="cuda")
    rc = fn(pts.data_ptr(), 5000, out.data_ptr(), 60, out.data_ptr(), out.data_ptr(), out.data_ptr(), None)
    assert rc == -2
    assert "4096" in lib.cuacd_last_error().decode()


def _entry(lib):
    fn = lib.cuacd_hull_points_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return fn


def test_no_alloc_refuses_a_triangle_buffer_a_hull_could_outgrow():
    torch = pytest.importorskip("torch")
    tree = importlib.import_module("cuacd-web_gb300.tree")
    gen = importlib.import_module("cuacd-web_gb300.meshgen")
    lib = tree.load_library()
    fn = _entry(lib)
    m = gen.noisy_icosphere(3, seed=4)  # 642 points: up to 1280 triangles
    pts = torch.from_numpy(np.ascontiguousarray(m.verts)).cuda()
    tris = torch.zeros(3 * (2 * m.nv - 4), dtype=torch.int32, device="cuda")
    res = torch.full((3,), -7, dtype=torch.int32, device="cuda")
    for cap in (12, 3 * (2 * m.nv - 4) - 1):
        rc = fn(pts.data_ptr(), m.nv, tris.data_ptr(), cap, res[0:].data_ptr(), res[1:].data_ptr(),
                res[2:].data_ptr(), None)
        assert rc == -2, rc
        assert str(3 * (2 * m.nv - 4)) in lib.cuacd_last_error().decode()
    torch.cuda.synchronize()
    assert res.tolist() == [-7, -7, -7]  # refused before any work was queued
    # the exact bound is accepted and gives the allocating entry point's hull
    rc = fn(pts.data_ptr(), m.nv, tris.data_ptr(), 3 * (2 * m.nv - 4), res[0:].data_ptr(), res[1:].data_ptr(),
            res[2:].data_ptr(), None)
    assert rc == 0, lib.cuacd_last_error().decode()
    torch.cuda.synchronize()
    g = tree.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, hullMaxVerts=4096)
    ref, st = g.hull_meshes([m])
    assert res[2].item() == 0 and st[0] == 0
    n = res[1].item()
    assert np.array_equal(tris[: 3 * n].cpu().numpy().astype(np.uint32).reshape(-1, 3), ref[0]["tris"])


def test_no_alloc_three_points_are_flat():
    torch = pytest.importorskip("torch")
    tree = importlib.import_module("cuacd-web_gb300.tree")
    lib = tree.load_library()
    fn = _entry(lib)
    pts = torch.tensor([0, 0, 0, 1, 0, 0, 0, 1, 0], dtype=torch.float32, device="cuda")
    tris = torch.full((12,), 5, dtype=torch.int32, device="cuda")
    vol = torch.full((1,), -3.0, dtype=torch.float32, device="cuda")
    nt = torch.full((1,), 99, dtype=torch.int32, device="cuda")
    st = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    rc = fn(pts.data_ptr(), 3, tris.data_ptr(), 12, vol.data_ptr(), nt.data_ptr(), st.data_ptr(), None)
    assert rc == 0, lib.cuacd_last_error().decode()
    torch.cuda.synchronize()
    assert st.item() == 8 and nt.item() == 0 and vol.item() == 0.0
