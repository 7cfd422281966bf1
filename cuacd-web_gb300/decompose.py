"""decompose(mesh, options) over libcuacd.so — the reference's public API
(src/decompose.ts:404-415, Decomposer at :128-392) with its options
(DecomposeOptions, :26-78) and result (DecomposeResult, :107-121).

The loop itself runs inside the library (csrc/decompose.cpp): the tree
search, capped cuts, concave-edge planes, hulls and Hausdorff distances on
the GPU, the merge pass's pairing and the output hulls' cleanup on host
threads. `decompose_batch` decomposes many
meshes in one call; with batched=True every iteration and merge round
serves all meshes with shared GPU launches, which gives the same parts as
decomposing them one at a time.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A
from .mesh import Mesh
from .tree import CuacdError, _check, load_library

# DEFAULT_OPTIONS (decompose.ts:83-106)
DEFAULT_OPTIONS = dict(
    threshold=0.05,
    maxIters=100,
    width=30,
    width2=3,
    depth=2,
    maxNCutting=16,
    nConcaveEdges=16,
    concaveEps=0.005,
    concaveThreshold=3.49,
    concaveIters=10,
    normalize=True,
    requireClosed=True,
    validateCuts=True,
    refineRounds=2,
    refineProbes=8,
    mergeHulls=True,
    mergeRounds=32,
    mergePlaneTol=1e-3,
    profile=False,
    threads=0,
    verbose=0,
    streams=1,
)

STUCK_REASONS = {0: None, 1: "no-plane", 2: "cut-failed", 3: "not-closed", 4: "degenerate"}

_bound = False


def _lib():
    global _bound
    L = load_library()
    if not _bound:
        P = C.POINTER
        L.cuacd_decompose_opts_default.argtypes = [P(A.DecomposeOpts)]
        L.cuacd_decomposer_create.restype = C.c_void_p
        L.cuacd_decomposer_create.argtypes = [P(A.DecomposeOpts), P(C.c_int)]
        L.cuacd_decomposer_destroy.argtypes = [C.c_void_p]
        L.cuacd_decompose.argtypes = [C.c_void_p, P(A.MeshRef), C.c_int, C.c_int, P(C.c_void_p)]
        L.cuacd_result_meshes.argtypes = [C.c_void_p]
        L.cuacd_result_parts.argtypes = [C.c_void_p, C.c_int]
        L.cuacd_result_part.argtypes = [C.c_void_p, C.c_int, C.c_int, P(A.PartView)]
        L.cuacd_result_stats.argtypes = [C.c_void_p, C.c_int, P(A.DecomposeStats)]
        L.cuacd_result_free.argtypes = [C.c_void_p]
        L.cuacd_plane_cut.argtypes = [P(A.MeshRef), P(C.c_double), P(C.c_void_p)]
        L.cuacd_cut_half.argtypes = [C.c_void_p, C.c_int, P(P(C.c_float)), P(C.c_uint32), P(P(C.c_uint32)),
                                     P(C.c_uint32)]
        L.cuacd_cut_free.argtypes = [C.c_void_p]
        L.cuacd_concave_planes.argtypes = [P(A.MeshRef), C.c_int, C.c_double, C.c_double, C.c_uint32, P(C.c_float),
                                           C.c_int]
        L.cuacd_server_create.restype = C.c_void_p
        L.cuacd_server_create.argtypes = [P(A.DecomposeOpts), C.c_uint64, C.c_int32, C.c_int32, P(C.c_int)]
        L.cuacd_server_stats.argtypes = [C.c_void_p, P(A.ServerStats)]
        L.cuacd_server_destroy.argtypes = [C.c_void_p]
        L.cuacd_server_submit.argtypes = [C.c_void_p, P(A.MeshRef), C.c_float, P(C.c_uint64)]
        L.cuacd_server_step.argtypes = [C.c_void_p, P(C.c_int)]
        L.cuacd_server_pending.argtypes = [C.c_void_p]
        L.cuacd_server_take.argtypes = [C.c_void_p, C.c_uint64, P(C.c_void_p)]
        L.cuacd_quickhull.argtypes = [P(C.c_double), C.c_int, C.c_double, P(C.c_double), C.c_int, P(C.c_uint32),
                                      C.c_int, P(C.c_int)]
        L.cuacd_clean_hull_faces.argtypes = [P(A.MeshRef), P(C.c_uint32), C.c_uint32, C.c_double, P(C.c_uint32),
                                             C.c_int]
        L.cuacd_merge_opts_default.argtypes = [P(A.MergeOpts)]
        L.cuacd_merge_hulls.argtypes = [C.c_void_p, P(A.PartIn), C.c_int, P(A.MergeOpts), P(C.c_void_p),
                                        P(A.MergeStats)]
        L.cuacd_seam_plane.argtypes = [P(A.PartIn), P(A.PartIn), C.c_double, P(C.c_double)]
        L.cuacd_filtered_concat.argtypes = [P(A.MeshRef), P(A.MeshRef), P(C.c_double), C.c_int, C.c_double,
                                            P(C.c_uint32), C.c_int]
        _bound = True
    return L


@dataclass
class Part:
    """Part (part.ts:9-22)."""

    mesh: Mesh
    hull: Mesh
    meshVol: float
    hullVol: float
    hausdorff: float | None
    stuck: bool = False
    stuckReason: str | None = None
    seams: list = field(default_factory=list)
    merged: int = 1


@dataclass
class DecomposeResult:
    """DecomposeResult (decompose.ts:107-121)."""

    parts: list
    iterations: int
    stats: dict


def _opts(kw) -> A.DecomposeOpts:
    L = _lib()
    o = A.DecomposeOpts()
    L.cuacd_decompose_opts_default(C.byref(o))
    tree = dict(kw.pop("tree", {}) or {})
    for k, v in kw.items():
        if k not in DEFAULT_OPTIONS:
            raise KeyError(f"unknown decompose option {k!r}")
        cur = getattr(o, k)
        setattr(o, k, float(v) if isinstance(cur, float) else int(v))
    for k, v in tree.items():
        if not hasattr(o.tree, k):
            raise KeyError(f"unknown tree config field {k!r}")
        setattr(o.tree, k, float(v) if k == "minEdgeDist" else int(v))
    return o


def _arr(ptr, n, dtype, width):
    if n == 0:
        return np.zeros((0, width), dtype)
    return np.ctypeslib.as_array(ptr, shape=(n * width,)).astype(dtype, copy=True).reshape(n, width)


def _take_results(res, n) -> list:
    """Copies n meshes' results out of a result handle and frees it."""
    L = _lib()
    try:
        out = []
        for k in range(n):
            parts = []
            for p in range(L.cuacd_result_parts(res, k)):
                v = A.PartView()
                _check(L.cuacd_result_part(res, k, p, C.byref(v)))
                seams = _arr(v.seams, v.nSeams, np.float64, 4)
                parts.append(Part(
                    mesh=Mesh(_arr(v.verts, v.nv, np.float32, 3), _arr(v.tris, v.nt, np.uint32, 3)),
                    hull=Mesh(_arr(v.hullVerts, v.hullNv, np.float32, 3), _arr(v.hullTris, v.hullNt, np.uint32, 3)),
                    meshVol=float(v.meshVol), hullVol=float(v.hullVol),
                    hausdorff=None if math.isnan(v.hausdorff) else float(v.hausdorff),
                    stuck=bool(v.stuck), stuckReason=STUCK_REASONS.get(v.stuckReason),
                    seams=[tuple(float(x) for x in s) for s in seams], merged=int(v.merged)))
            st = A.DecomposeStats()
            _check(L.cuacd_result_stats(res, k, C.byref(st)))
            stats = {name: getattr(st, name) for name, _ in A.DecomposeStats._fields_}
            out.append(DecomposeResult(parts=parts, iterations=int(st.iterations), stats=stats))
        return out
    finally:
        L.cuacd_result_free(res)


class Decomposer:
    """Decomposer (decompose.ts:128-392): one GPU tree, reused across calls."""

    def __init__(self, **options):
        L = _lib()
        self.opts = _opts(dict(options))
        err = C.c_int(0)
        self.h = L.cuacd_decomposer_create(C.byref(self.opts), C.byref(err))
        if not self.h:
            raise CuacdError(err.value, L.cuacd_last_error().decode())

    def destroy(self):
        if getattr(self, "h", None):
            _lib().cuacd_decomposer_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def decompose_many(self, meshes, batched: bool = True) -> list:
        L = _lib()
        ma = A.MeshArray([A.as_mesh(m) for m in meshes])
        res = C.c_void_p()
        _check(L.cuacd_decompose(self.h, ma.arr, ma.n, int(batched), C.byref(res)))
        return _take_results(res, ma.n)

    def decompose(self, mesh) -> DecomposeResult:
        return self.decompose_many([mesh], batched=False)[0]


    def merge_hulls(self, parts, threshold: float = 0.05, max_rounds: int = 32, plane_tol: float = 1e-3,
                    hull_eps: float = 2e-5, verbose: int = 0):
        """mergeHulls(tree, parts, opts) (merge.ts:170-303) on this
        decomposer's GPU tree: returns (merged parts, MergeStats dict)."""
        L = _lib()
        mo = A.MergeOpts()
        L.cuacd_merge_opts_default(C.byref(mo))
        mo.threshold, mo.maxRounds, mo.planeTol, mo.hullEps, mo.verbose = threshold, max_rounds, plane_tol, hull_eps, verbose
        pa = A.PartArray(parts)
        res = C.c_void_p()
        st = A.MergeStats()
        _check(L.cuacd_merge_hulls(self.h, pa.arr, pa.n, C.byref(mo), C.byref(res), C.byref(st)))
        out = _take_results(res, 1)[0]
        return out.parts, {name: getattr(st, name) for name, _ in A.MergeStats._fields_ if name != "reserved"}


def merge_hulls(parts, threshold: float = 0.05, max_rounds: int = 32, plane_tol: float = 1e-3, hull_eps: float = 2e-5,
                **options):
    """mergeHulls (merge.ts:170-303): (merged parts, MergeStats dict)."""
    d = Decomposer(threshold=threshold, **options)
    try:
        return d.merge_hulls(parts, threshold, max_rounds, plane_tol, hull_eps)
    finally:
        d.destroy()


def seam_plane(a, b, tol: float = 1e-3):
    """seamPlane (merge.ts:114-141): the plane (a, b, c, d) or None."""
    pa = A.PartArray([a, b])
    out = (C.c_double * 4)()
    rc = _lib().cuacd_seam_plane(C.byref(pa.arr[0]), C.byref(pa.arr[1]), float(tol), out)
    if rc < 0:
        _check(rc)
    return tuple(float(x) for x in out) if rc == 1 else None


def filtered_concat(a, b, planes, tol: float = 1e-3) -> Mesh:
    """filteredConcat (merge.ts:144-157): the concatenation of a and b without
    the triangles lying on any of the planes."""
    ma = A.MeshArray([A.as_mesh(a), A.as_mesh(b)])
    pl = np.ascontiguousarray(np.asarray(planes, np.float64).reshape(-1, 4))
    cap = a.nt + b.nt
    out = np.zeros(max(3 * cap, 3), np.uint32)
    n = _lib().cuacd_filtered_concat(C.byref(ma.arr[0]), C.byref(ma.arr[1]), pl.ctypes.data_as(C.POINTER(C.c_double)),
                                     pl.shape[0], float(tol), A.uptr(out), cap)
    if n < 0:
        _check(n)
    return Mesh(np.concatenate([a.verts, b.verts]).astype(np.float32), out[: 3 * n].reshape(-1, 3).copy())


def decompose(mesh, **options) -> DecomposeResult:
    """decompose(mesh, opts) (decompose.ts:404-415)."""
    d = Decomposer(**options)
    try:
        return d.decompose(mesh)
    finally:
        d.destroy()


def decompose_batch(meshes, batched: bool = True, **options) -> list:
    """Decomposes many meshes in one call (same parts as one at a time)."""
    d = Decomposer(**options)
    try:
        return d.decompose_many(meshes, batched=batched)
    finally:
        d.destroy()


class Server:
    """Continuous batching of decompositions (cuacd_server_*): submit
    meshes at any time, step the server, take finished results. Each step
    runs one iteration of every admitted decomposition together; requests
    are admitted in arrival order while one of max_active slots is free (0:
    no bound) and the server's device memory, with its pools grown for every
    admitted request's working set, stays within admit_bytes (0: 80 % of the
    device's memory). At most max_queue requests wait (0: no bound); submit
    raises CuacdError with CUACD_E_BUSY (-6) when the queue is full."""

    E_BUSY = -6

    def __init__(self, admit_bytes: int = 0, max_active: int = 0, max_queue: int = 0, **options):
        L = _lib()
        self.opts = _opts(dict(options))
        err = C.c_int(0)
        self.h = L.cuacd_server_create(C.byref(self.opts), C.c_uint64(int(admit_bytes)), C.c_int32(int(max_active)),
                                       C.c_int32(int(max_queue)), C.byref(err))
        if not self.h:
            raise CuacdError(err.value, L.cuacd_last_error().decode())

    def stats(self) -> dict:
        """Device budget and bytes held, working sets, admitted / rejected
        counts and queue lengths (cuacd_server_stats)."""
        st = A.ServerStats()
        _check(_lib().cuacd_server_stats(self.h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in A.ServerStats._fields_}

    def destroy(self):
        if getattr(self, "h", None):
            _lib().cuacd_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def submit(self, mesh, threshold: float = 0.0) -> int:
        ma = A.MeshArray([A.as_mesh(mesh)])
        t = C.c_uint64()
        _check(_lib().cuacd_server_submit(self.h, ma.arr, C.c_float(threshold), C.byref(t)))
        return int(t.value)

    def step(self) -> int:
        n = C.c_int(0)
        _check(_lib().cuacd_server_step(self.h, C.byref(n)))
        return int(n.value)

    @property
    def pending(self) -> int:
        return int(_lib().cuacd_server_pending(self.h))

    def take(self, ticket: int):
        """The DecomposeResult of a finished request, or None while it runs."""
        res = C.c_void_p()
        rc = _lib().cuacd_server_take(self.h, C.c_uint64(ticket), C.byref(res))
        if rc == 1:
            return None
        _check(rc)
        return _take_results(res, 1)[0]


def plane_cut(mesh, plane):
    """planeCut with caps (src/cpu/cut.ts:33-315) on the library's host path.
    Returns (pos, neg) meshes, or raises CuacdError with the reference's
    reason when the cut fails."""
    L = _lib()
    ma = A.MeshArray([A.as_mesh(mesh)])
    pl = (C.c_double * 4)(*[float(x) for x in plane])
    h = C.c_void_p()
    _check(L.cuacd_plane_cut(ma.arr, pl, C.byref(h)))
    try:
        out = []
        for side in (0, 1):
            v = C.POINTER(C.c_float)()
            t = C.POINTER(C.c_uint32)()
            nv = C.c_uint32()
            nt = C.c_uint32()
            _check(L.cuacd_cut_half(h, side, C.byref(v), C.byref(nv), C.byref(t), C.byref(nt)))
            out.append(Mesh(_arr(v, nv.value, np.float32, 3), _arr(t, nt.value, np.uint32, 3)))
        return out[0], out[1]
    finally:
        L.cuacd_cut_free(h)


def concave_planes(mesh, n_concave_edges=16, concave_eps=0.005, concave_threshold=3.49, seed=12345) -> np.ndarray:
    """concaveEdgePlanes (src/cpu/concave.ts:25-92) on the library's host
    path: (n, 4) float32 planes."""
    L = _lib()
    ma = A.MeshArray([A.as_mesh(mesh)])
    cap = 4 * max(n_concave_edges, 0)
    out = np.zeros(max(4 * cap, 4), np.float32)
    n = L.cuacd_concave_planes(ma.arr, int(n_concave_edges), float(concave_eps), float(concave_threshold),
                               int(seed) & 0xFFFFFFFF, A.fptr(out), cap)
    if n < 0:
        _check(n)
    return out[: 4 * min(n, cap)].reshape(-1, 4).copy()


def quickhull(points, eps: float = 1e-7):
    """The reference's CPU hull, qh_compute (wasm/qh.cpp:16-25): returns
    (vertices (m, 3) float64, triangles (k, 3) uint32), vertices in first
    appearance order, triangles counter-clockwise seen from outside."""
    L = _lib()
    p = np.ascontiguousarray(np.asarray(points, np.float64).reshape(-1, 3))
    n = p.shape[0]
    vcap, tcap = max(n, 4), max(2 * n, 4)
    v = np.zeros(3 * vcap, np.float64)
    t = np.zeros(3 * tcap, np.uint32)
    nv = C.c_int(0)
    dp = C.POINTER(C.c_double)
    k = L.cuacd_quickhull(p.ctypes.data_as(dp), n, float(eps), v.ctypes.data_as(dp), vcap,
                          t.ctypes.data_as(C.POINTER(C.c_uint32)), tcap, C.byref(nv))
    if k < 0:
        _check(k)
    return v[: 3 * nv.value].reshape(-1, 3).copy(), t[: 3 * k].reshape(-1, 3).copy()


def clean_hull_faces(verts, tris, eps: float = 2e-5) -> np.ndarray:
    """cleanHullFaces (src/cpu/hull.ts:87-155): hull triangles (indices into
    verts) rebuilt for output; the input triangles when the rebuild is not
    accepted."""
    L = _lib()
    v = np.ascontiguousarray(np.asarray(verts, np.float32).reshape(-1, 3))
    t = np.ascontiguousarray(np.asarray(tris, np.uint32).reshape(-1, 3))
    ma = A.MeshArray([Mesh(v, np.zeros((0, 3), np.uint32))])
    cap = max(2 * v.shape[0], t.shape[0], 1)
    out = np.zeros(3 * cap, np.uint32)
    up = C.POINTER(C.c_uint32)
    k = L.cuacd_clean_hull_faces(ma.arr, t.ctypes.data_as(up), t.shape[0], float(eps), out.ctypes.data_as(up), cap)
    if k < 0:
        _check(k)
    return out[: 3 * k].reshape(-1, 3).copy()
