"""ctypes harness over the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: the oracle is the checker for the CUDA engine and
is loaded only by tests, __graft_entry__.smoke() and bench.py's CPU-baseline
leg. It shares the engine's ctypes struct mirrors (the same C layouts) and
nothing else.
"""
from __future__ import annotations

import ctypes as C
import importlib
import os
import subprocess
import sys

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(ORACLE_DIR)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
A = importlib.import_module("cuacd-web_gb300._abi")
Mesh = importlib.import_module("cuacd-web_gb300.mesh").Mesh
_lib = None


def reference_dir():
    """The reference checkout, where present (CUACD_REFERENCE_DIR)."""
    return os.environ.get("CUACD_REFERENCE_DIR", "/root/reference")


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "liboracle.so"], check=True)
    if os.path.exists(os.path.join(reference_dir(), "wasm/quickhull/QuickHull.cpp")):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref"], check=True)


def lib():
    global _lib
    if _lib is not None:
        return _lib
    path = os.path.join(ORACLE_DIR, "liboracle.so")
    if not os.path.exists(path):
        build_oracle()
    L = C.CDLL(path)
    P = C.POINTER
    L.orc_tree_create.restype = C.c_void_p
    L.orc_tree_create.argtypes = [P(A.TreeConfig)]
    L.orc_tree_destroy.argtypes = [C.c_void_p]
    L.orc_plane_slots.argtypes = [C.c_void_p]
    L.orc_tree_run.argtypes = [C.c_void_p, P(A.MeshRef), C.c_int, P(C.c_float), C.c_int, P(A.RunOpts),
                               P(A.SeedResult), P(A.RunStats)]
    L.orc_tree_hull_meshes.argtypes = [C.c_void_p, P(A.MeshRef), C.c_int, C.c_int, C.c_int, P(C.c_uint32),
                                       C.c_uint32, P(C.c_float), P(C.c_uint32), P(C.c_int32)]
    for f in ("orc_read_items", "orc_read_parts", "orc_read_jobs"):
        getattr(L, f).argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, P(C.c_uint32)]
    L.orc_read_part_geometry.argtypes = [C.c_void_p, C.c_uint32, P(C.c_float), P(C.c_uint32), P(C.c_uint32)]
    L.orc_read_plane.argtypes = [C.c_void_p, C.c_uint32, P(C.c_float)]
    L.orc_last_items.restype = C.c_uint32
    L.orc_last_items.argtypes = [C.c_void_p]
    L.orc_last_error.restype = C.c_char_p
    L.orc_hausdorff_gpu.argtypes = [P(A.MeshRef), P(A.MeshRef), C.c_int, P(C.c_uint32), P(C.c_float)]
    L.orc_hausdorff_cpu.argtypes = [P(A.MeshRef), P(A.MeshRef), C.c_int, P(C.c_double)]
    L.orc_sample_gpu.argtypes = [P(A.MeshRef), C.c_uint32, P(C.c_float), C.c_uint32]
    L.orc_signed_volume.restype = C.c_double
    L.orc_signed_volume.argtypes = [P(A.MeshRef)]
    L.orc_is_closed.argtypes = [P(A.MeshRef)]
    L.orc_plane_cut.argtypes = [P(A.MeshRef), P(C.c_double), P(C.c_float), P(C.c_uint32), P(C.c_float),
                                P(C.c_uint32), C.c_uint32, C.c_uint32, P(C.c_uint32)]
    L.orc_concave_planes.argtypes = [P(A.MeshRef), C.c_int, C.c_double, C.c_double, C.c_uint32, P(C.c_float), C.c_int]
    L.orc_hull_volume.restype = C.c_double
    L.orc_hull_volume.argtypes = [P(A.MeshRef), C.c_int]
    L.orc_rv_cost.restype = C.c_float
    L.orc_rv_cost.argtypes = [C.c_float, C.c_float]
    L.orc_eval_candidates.argtypes = [P(A.MeshRef), P(C.c_double), C.c_int, C.c_int, C.c_int, C.c_int, P(C.c_double)]
    L.orc_load_qh_ref.argtypes = [C.c_char_p]
    L.orc_seam_plane.argtypes = [P(A.PartIn), P(A.PartIn), C.c_double, P(C.c_double)]
    L.orc_filtered_concat.argtypes = [P(A.MeshRef), P(A.MeshRef), P(C.c_double), C.c_int, C.c_double, P(C.c_uint32),
                                      C.c_int]
    L.orc_merge_hulls.argtypes = [P(A.PartIn), C.c_int, C.c_double, C.c_int, C.c_double, P(C.c_int), P(C.c_int),
                                  P(C.c_int), P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_int), P(C.c_int)]
    ref = os.path.join(ORACLE_DIR, "_ref", "libqh_ref.so")
    if os.path.exists(ref):
        try:
            L.orc_load_qh_ref(ref.encode())
        except OSError:
            pass
    _lib = L
    return L


def qh_ref_loaded() -> bool:
    return bool(lib().orc_qh_ref_loaded())


class OracleTree:
    """CPU restatement of GpuTree (src/gpu/tree.ts) with the engine's interface."""

    def __init__(self, **cfg):
        self.cfg = A.make_config(**cfg)
        self.h = lib().orc_tree_create(C.byref(self.cfg))
        if not self.h:
            raise ValueError(lib().orc_last_error().decode())
        self.plane_slots = lib().orc_plane_slots(self.h)

    def destroy(self):
        if self.h:
            lib().orc_tree_destroy(self.h)
            self.h = None

    def __del__(self):
        self.destroy()

    def run(self, seeds, edge_planes=None, depth=0, width=-1, n_edge_cuts=-1, refine=None):
        seeds = [A.as_mesh(s) for s in seeds]
        ma = A.MeshArray(seeds)
        n = len(seeds)
        k = self.plane_slots
        ep = np.zeros((max(n, 1), k, 4), np.float32)
        if edge_planes is not None:
            for i, p in enumerate(edge_planes):
                if p is None:
                    continue
                p = np.asarray(p, np.float32).reshape(-1, 4)[:k]
                ep[i, : len(p)] = p
        opts = A.RunOpts(depth=depth, width=width, nEdgeCuts=n_edge_cuts)
        spacing = None
        if refine:
            opts.refineRounds = refine["rounds"]
            opts.refineProbes = refine["probes"]
            spacing = np.asarray(refine["spacing"], np.float32)
            opts.refineSpacing = A.fptr(spacing)
        out = (A.SeedResult * max(n, 1))()
        st = A.RunStats()
        rc = lib().orc_tree_run(self.h, ma.arr, n, A.fptr(ep), k, C.byref(opts), out, C.byref(st))
        if rc != 0:
            raise ValueError(lib().orc_last_error().decode())
        return _result(out, st, n)

    def hull_meshes(self, meshes, hull_stage=0, no_export=False):
        meshes = [A.as_mesh(m) for m in meshes]
        ma = A.MeshArray(meshes)
        n = len(meshes)
        maxnv = max(m.nv for m in meshes)
        stride = 3 * 2 * min(self.cfg.hullMaxVerts, maxnv)
        tris = np.zeros(n * stride, np.uint32)
        vol = np.zeros(n, np.float32)
        nt = np.zeros(n, np.uint32)
        status = np.zeros(n, np.int32)
        rc = lib().orc_tree_hull_meshes(self.h, ma.arr, n, hull_stage, int(no_export), A.uptr(tris), stride,
                                        A.fptr(vol), A.uptr(nt), status.ctypes.data_as(C.POINTER(C.c_int32)))
        if rc != 0:
            raise ValueError(lib().orc_last_error().decode())
        out = []
        for i in range(n):
            if status[i] != 0:
                out.append(None)
            else:
                out.append(dict(tris=tris[i * stride: i * stride + 3 * nt[i]].reshape(-1, 3).copy(), volume=float(vol[i])))
        return out, status

    def items(self, first, n):
        w = np.zeros(20 * n, np.uint32)
        assert lib().orc_read_items(self.h, first, n, A.uptr(w)) == 0
        return w.reshape(n, 20)

    def parts(self, first, n):
        w = np.zeros(16 * n, np.uint32)
        assert lib().orc_read_parts(self.h, first, n, A.uptr(w)) == 0
        return w.reshape(n, 16)

    def jobs(self, first, n):
        w = np.zeros(24 * n, np.uint32)
        assert lib().orc_read_jobs(self.h, first, n, A.uptr(w)) == 0
        return w.reshape(n, 24)

    def part_geometry(self, idx):
        d = self.parts(idx, 1)[0]
        v = np.zeros(3 * d[1], np.float32)
        t = np.zeros(3 * d[3], np.uint32)
        e = np.zeros(8 * d[5], np.uint32)
        lib().orc_read_part_geometry(self.h, idx, A.fptr(v), A.uptr(t), A.uptr(e))
        return v.reshape(-1, 3), t.reshape(-1, 3), e.reshape(-1, 8)

    def plane(self, idx):
        f = np.zeros(4, np.float32)
        lib().orc_read_plane(self.h, idx, A.fptr(f))
        return f


def _result(out, st, n):
    seeds = []
    for i in range(n):
        s = out[i]
        seeds.append(dict(bestCut=s.bestCut, bestCost=s.bestCost if s.valid else float("inf"),
                          plane=list(s.plane) if s.valid else None))
    return dict(
        seeds=seeds, overflow=bool(st.overflow), hullFail=bool(st.hullFail), hullFailCount=st.hullFailCount,
        npOverflow=bool(st.npOverflow), pruned=st.pruned, jobsPerLevel=list(st.jobsPerLevel[: st.nLevels]),
        validJobs=st.validJobs, hullSlabWords=st.hullSlabWords,
    )


def hausdorff_gpu_form(pairs, caps=None):
    a = A.MeshArray([A.as_mesh(p[0]) for p in pairs])
    b = A.MeshArray([A.as_mesh(p[1]) for p in pairs])
    out = np.zeros(len(pairs), np.float32)
    cp = None
    if caps is not None:
        caps = np.asarray(caps, np.uint32)
        cp = A.uptr(caps)
    lib().orc_hausdorff_gpu(a.arr, b.arr, len(pairs), cp, A.fptr(out))
    return out


def hausdorff_cpu(a, b) -> float:
    ma, mb = A.MeshArray([A.as_mesh(a)]), A.MeshArray([A.as_mesh(b)])
    out = np.zeros(1, np.float64)
    lib().orc_hausdorff_cpu(ma.arr, mb.arr, 1, out.ctypes.data_as(C.POINTER(C.c_double)))
    return float(out[0])


def sample_gpu_form(m, cap=0):
    ma = A.MeshArray([A.as_mesh(m)])
    n = lib().orc_sample_gpu(ma.arr, cap, None, 0)
    out = np.zeros(3 * max(n, 1), np.float32)
    lib().orc_sample_gpu(ma.arr, cap, A.fptr(out), n)
    return out[: 3 * n].reshape(-1, 3)


def plane_cut(m, plane):
    m = A.as_mesh(m)
    ma = A.MeshArray([m])
    cap_v = 4 * m.nv + 4 * m.nt + 64
    cap_t = 8 * m.nt + 64
    pv, nvv = np.zeros(3 * cap_v, np.float32), np.zeros(3 * cap_v, np.float32)
    pt, ntt = np.zeros(3 * cap_t, np.uint32), np.zeros(3 * cap_t, np.uint32)
    cnt = np.zeros(4, np.uint32)
    pl = np.asarray(plane, np.float64)
    rc = lib().orc_plane_cut(ma.arr, pl.ctypes.data_as(C.POINTER(C.c_double)), A.fptr(pv), A.uptr(pt), A.fptr(nvv),
                             A.uptr(ntt), cap_v, cap_t, A.uptr(cnt))
    if rc != 0:
        return None
    pos = Mesh(pv[: 3 * cnt[0]], pt[: 3 * cnt[1]])
    neg = Mesh(nvv[: 3 * cnt[2]], ntt[: 3 * cnt[3]])
    return pos, neg


def concave_planes(m, n_concave_edges=16, eps=0.005, thresh=3.49, seed=12345):
    m = A.as_mesh(m)
    ma = A.MeshArray([m])
    cap = 4 * max(n_concave_edges, 1)
    out = np.zeros(4 * cap, np.float32)
    n = lib().orc_concave_planes(ma.arr, n_concave_edges, eps, thresh, seed, A.fptr(out), cap)
    return out[: 4 * min(n, cap)].reshape(-1, 4)


def hull_volume(m, use_ref=True) -> float:
    ma = A.MeshArray([A.as_mesh(m)])
    return float(lib().orc_hull_volume(ma.arr, int(use_ref)))


def is_closed(m) -> bool:
    ma = A.MeshArray([A.as_mesh(m)])
    return bool(lib().orc_is_closed(ma.arr))


def rv_cost(mv, hv) -> float:
    return float(lib().orc_rv_cost(mv, hv))


def eval_candidates(m, planes, threads=1, with_hd=True, use_ref=True):
    ma = A.MeshArray([A.as_mesh(m)])
    pl = np.ascontiguousarray(np.asarray(planes, np.float64).reshape(-1, 4))
    out = np.zeros((len(pl), 8), np.float64)
    lib().orc_eval_candidates(ma.arr, pl.ctypes.data_as(C.POINTER(C.c_double)), len(pl), threads, int(with_hd),
                              int(use_ref), out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


# ---- the reference's own CPU hull (oracle/_ref/libqh_ref.so) ----------------

_qh = None


def qh_ref():
    """ctypes handle of the reference's quickhull compiled from its sources
    (None when oracle/_ref was not built: it needs the reference tree)."""
    global _qh
    if _qh is None:
        path = os.path.join(ORACLE_DIR, "_ref", "libqh_ref.so")
        if not os.path.exists(path):
            return None
        L = C.CDLL(path)
        P = C.POINTER
        L.qhref_compute.argtypes = [P(C.c_double), C.c_int, C.c_double, P(C.c_double), C.c_int, P(C.c_uint32),
                                    C.c_int, P(C.c_int)]
        _qh = L
    return _qh


def quickhull_ref(points, eps=1e-7):
    """qh_compute (wasm/qh.cpp:16-25) on the reference's quickhull:
    (vertices (m, 3) float64, triangles (k, 3) uint32)."""
    L = qh_ref()
    p = np.ascontiguousarray(np.asarray(points, np.float64).reshape(-1, 3))
    n = p.shape[0]
    vcap, tcap = max(n, 4), max(2 * n, 4)
    v = np.zeros(3 * vcap, np.float64)
    t = np.zeros(3 * tcap, np.uint32)
    nv = C.c_int(0)
    dp = C.POINTER(C.c_double)
    k = L.qhref_compute(p.ctypes.data_as(dp), n, float(eps), v.ctypes.data_as(dp), vcap,
                        t.ctypes.data_as(C.POINTER(C.c_uint32)), tcap, C.byref(nv))
    assert k >= 0
    return v[: 3 * nv.value].reshape(-1, 3).copy(), t[: 3 * k].reshape(-1, 3).copy()


def _signed_volume_js(V, T):
    # src/mesh.ts:59-72, anchored at vertex 0 of V, in double
    if len(T) == 0:
        return 0.0
    o = V[0].astype(np.float64)
    s = 0.0
    for a, b, c in T:
        A = V[a].astype(np.float64) - o
        B = V[b].astype(np.float64) - o
        Cc = V[c].astype(np.float64) - o
        s += A[0] * (B[1] * Cc[2] - B[2] * Cc[1]) + A[1] * (B[2] * Cc[0] - B[0] * Cc[2]) + A[2] * (B[0] * Cc[1] - B[1] * Cc[0])
    return s / 6


def _closed_js(T, nv):
    # src/mesh.ts:104-119: every directed edge once, its reverse once
    cnt = {}
    for t in T:
        for e in range(3):
            a, b = int(t[e]), int(t[(e + 1) % 3])
            if a >= nv or b >= nv:
                return False
            cnt[(a, b)] = cnt.get((a, b), 0) + 1
    return all(c == 1 and cnt.get((b, a)) == 1 for (a, b), c in cnt.items())


def clean_hull_faces_ref(V, T, eps=2e-5):
    """cleanHullFaces (src/cpu/hull.ts:87-155) restated in Python over the
    reference's quickhull. V (n, 3) float32, T (k, 3) indices."""
    import math
    V = np.asarray(V, np.float32).reshape(-1, 3)
    T = np.asarray(T, np.uint32).reshape(-1, 3)
    if T.size < 12:
        return T
    cand, seen = [], set()
    for x in T.reshape(-1):
        if int(x) not in seen:
            seen.add(int(x))
            cand.append(int(x))
    vraw = abs(_signed_volume_js(V, T))
    vals = [float(V[c][a]) for c in cand for a in range(3)]
    extent = max(max(vals) - min(vals), 1e-30)
    tol = 5 * eps * extent
    for _ in range(6):
        n = len(cand)
        if n < 4:
            return T
        pts = np.array([[float(x) for x in V[c]] for c in cand], np.float64)
        by_key = {}
        for k, c in enumerate(cand):
            by_key[tuple(pts[k])] = c
        hv, ht = quickhull_ref(pts, eps)
        out = []
        for tri in ht:
            row = []
            for i in tri:
                key = tuple(hv[i])
                if key not in by_key:
                    return T
                row.append(by_key[key])
            out.append(row)
        out = np.array(out, np.uint32).reshape(-1, 3)
        if not _closed_js(out, V.shape[0]):
            return T
        sv = _signed_volume_js(V, out)
        if sv < 0:
            out = out[:, [0, 2, 1]]
        if not (abs(abs(sv) - vraw) <= 10 * eps * vraw + 1e-30):
            return T
        drop = []
        for ia, ib, ic in out:
            a, b, c = (V[i].astype(np.float64) for i in (ia, ib, ic))
            u, w = b - a, c - a
            nx, ny, nz = u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]
            l = math.hypot(nx, ny, nz)
            lab, lac, lbc = math.hypot(*u), math.hypot(*w), math.hypot(*(c - b))
            longest = max(lab, lac, lbc)
            if not (l > eps * extent * longest):
                d = ia if (lbc >= lab and lbc >= lac) else (ib if lac >= lab else ic)
                if int(d) not in drop:
                    drop.append(int(d))
                continue
            nx, ny, nz = nx / l, ny / l, nz / l
            d = nx * a[0] + ny * a[1] + nz * a[2]
            for q in cand:
                p = V[q].astype(np.float64)
                if nx * p[0] + ny * p[1] + nz * p[2] - d > tol:
                    return T
        if not drop:
            return out
        cand = [c for c in cand if c not in drop]
    return T


# ---- the merge pass (merge_oracle.cpp) ----------------------------------------

def seam_plane(a, b, tol=1e-3):
    """seamPlane (merge.ts:114-141): the plane (a, b, c, d) or None."""
    pa = A.PartArray([a, b])
    out = (C.c_double * 4)()
    ok = lib().orc_seam_plane(C.byref(pa.arr[0]), C.byref(pa.arr[1]), float(tol), out)
    return tuple(float(x) for x in out) if ok else None


def filtered_concat(a, b, planes, tol=1e-3):
    """filteredConcat (merge.ts:144-157): kept triangles over a's then b's vertices."""
    ma = A.MeshArray([A.as_mesh(a), A.as_mesh(b)])
    pl = np.ascontiguousarray(np.asarray(planes, np.float64).reshape(-1, 4))
    cap = a.nt + b.nt
    out = np.zeros(max(3 * cap, 3), np.uint32)
    n = lib().orc_filtered_concat(C.byref(ma.arr[0]), C.byref(ma.arr[1]), pl.ctypes.data_as(C.POINTER(C.c_double)),
                                  pl.shape[0], float(tol), A.uptr(out), cap)
    return out[: 3 * n].reshape(-1, 3).copy()


def merge_hulls(parts, threshold=0.05, max_rounds=32, plane_tol=1e-3):
    """mergeHulls (merge.ts:170-303) on the oracle's grid hull and float32
    Hausdorff: a list of output parts (members = input parts in
    concatenation order, meshVol, hullVol, hausdorff, nSeams) and the stats
    (rounds, merges, pairsHulled, pairsHausdorff)."""
    n = len(parts)
    pa = A.PartArray(parts)
    n_out = C.c_int(0)
    ms = np.zeros(n + 1, np.int32)
    mem = np.zeros(max(n, 1), np.int32)
    mv, hv, hd = np.zeros(max(n, 1)), np.zeros(max(n, 1)), np.zeros(max(n, 1))
    ns = np.zeros(max(n, 1), np.int32)
    st = np.zeros(4, np.int32)
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    lib().orc_merge_hulls(pa.arr, n, float(threshold), int(max_rounds), float(plane_tol), C.byref(n_out), ip(ms),
                          ip(mem), dp(mv), dp(hv), dp(hd), ip(ns), ip(st))
    out = [dict(members=mem[ms[k]:ms[k + 1]].tolist(), meshVol=float(mv[k]), hullVol=float(hv[k]),
                hausdorff=float(hd[k]), nSeams=int(ns[k])) for k in range(n_out.value)]
    return out, dict(rounds=int(st[0]), merges=int(st[1]), pairsHulled=int(st[2]), pairsHausdorff=int(st[3]))
