"""GpuTree over libcuacd.so — the reference's GpuTree (src/gpu/tree.ts) on the
GB300 engine.

Method names follow the reference: run, hausdorff, hull_meshes,
hulls_with_hausdorff, plane_slots, read_part, read_plane; table readers
return the reference's word layouts. There is no fallback: if libcuacd.so is
missing or no CUDA device is present, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi as A
from .mesh import Mesh, mesh_area

HERE = os.path.dirname(os.path.abspath(__file__))
HD_MAX_PAIRS = 1024
_lib = None


class CuacdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"cuacd error {code}: {msg}")
        self.code = code


class ScratchError(CuacdError):
    """Hausdorff sample scratch exceeded. The message contains "scratch", as
    the reference's Error does (tree.ts:345), so merge-style callers can halve
    the batch on it (merge.ts:405)."""


def library_path() -> str:
    return os.path.join(HERE, "libcuacd.so")


def load_library():
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with __graft_entry__.build() or cuacd-web_gb300/build.py")
    L = C.CDLL(path)
    P = C.POINTER
    L.cuacd_last_error.restype = C.c_char_p
    L.cuacd_tree_config_default.argtypes = [P(A.TreeConfig)]
    L.cuacd_tree_create.restype = C.c_void_p
    L.cuacd_tree_create.argtypes = [P(A.TreeConfig), P(C.c_int)]
    L.cuacd_tree_destroy.argtypes = [C.c_void_p]
    L.cuacd_plane_slots.argtypes = [C.c_void_p]
    L.cuacd_device_memory.argtypes = [P(C.c_uint64), P(C.c_uint64)]
    L.cuacd_tree_memory.argtypes = [C.c_void_p, P(C.c_uint64), P(C.c_uint64)]
    L.cuacd_tree_reserve_pools.argtypes = [C.c_void_p, P(C.c_uint64)]
    L.cuacd_tree_schedule.argtypes = [C.c_void_p, P(C.c_int32)]
    L.cuacd_set_profile.argtypes = [C.c_void_p, C.c_int]
    L.cuacd_tree_kernel_ms.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
    L.cuacd_tree_kernel_bytes.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
    L.cuacd_tree_hd_stats.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
    L.cuacd_tree_last_gpu_ms.restype = C.c_float
    L.cuacd_tree_last_gpu_ms.argtypes = [C.c_void_p]
    run_args = [C.c_void_p, P(A.MeshRef), C.c_int, P(C.c_float), C.c_int, P(A.RunOpts)]
    L.cuacd_tree_run.argtypes = run_args + [P(A.SeedResult), P(A.RunStats)]
    L.cuacd_tree_prepare.argtypes = run_args
    L.cuacd_tree_launch.argtypes = [C.c_void_p]
    L.cuacd_tree_collect.argtypes = [C.c_void_p, P(A.SeedResult), P(A.RunStats)]
    L.cuacd_tree_hausdorff.argtypes = [C.c_void_p, P(A.MeshRef), P(A.MeshRef), C.c_int, P(C.c_float)]
    L.cuacd_tree_hull_meshes.argtypes = [C.c_void_p, P(A.MeshRef), C.c_int, C.c_int, P(C.c_uint32), C.c_uint32,
                                         P(C.c_float), P(C.c_uint32), P(C.c_int32)]
    L.cuacd_tree_hulls_with_hausdorff.argtypes = [C.c_void_p, P(A.MeshRef), C.c_int, P(C.c_uint32), C.c_uint32,
                                                  P(C.c_float), P(C.c_uint32), P(C.c_float), P(C.c_int32)]
    for f in ("cuacd_tree_read_items", "cuacd_tree_read_parts", "cuacd_tree_read_jobs"):
        getattr(L, f).argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, P(C.c_uint32)]
    L.cuacd_tree_read_part_geometry.argtypes = [C.c_void_p, C.c_uint32, P(C.c_float), P(C.c_uint32), P(C.c_uint32)]
    L.cuacd_tree_read_plane.argtypes = [C.c_void_p, C.c_uint32, P(C.c_float)]
    L.cuacd_tree_plane_cuts.argtypes = [C.c_void_p, P(A.MeshRef), C.c_int, P(C.c_int32), P(C.c_double), C.c_int,
                                        C.c_int, P(C.c_void_p)]
    L.cuacd_cuts_half.argtypes = [C.c_void_p, C.c_int, C.c_int, P(P(C.c_float)), P(C.c_uint32), P(P(C.c_uint32)),
                                  P(C.c_uint32)]
    L.cuacd_cuts_gpu_ms.restype = C.c_float
    L.cuacd_cuts_gpu_ms.argtypes = [C.c_void_p]
    L.cuacd_cuts_free.argtypes = [C.c_void_p]
    L.cuacd_tree_concave_planes.argtypes = [C.c_void_p, P(A.MeshRef), C.c_int, C.c_int, C.c_double, C.c_double,
                                            P(C.c_uint32), P(C.c_float), P(C.c_int32)]
    L.cuacd_tree_concave_ms.restype = C.c_float
    L.cuacd_tree_concave_ms.argtypes = [C.c_void_p]
    L.cuacd_tree_eval_cuts.argtypes = [C.c_void_p, P(A.MeshRef), P(C.c_double), C.c_int, P(C.c_double)]
    L.cuacd_tree_eval_cuts_ms.restype = C.c_float
    L.cuacd_tree_eval_cuts_ms.argtypes = [C.c_void_p]
    _lib = L
    return L


def device_memory():
    """(total, free) bytes of the current device (cudaMemGetInfo)."""
    tot, free = C.c_uint64(), C.c_uint64()
    _check(load_library().cuacd_device_memory(C.byref(tot), C.byref(free)))
    return tot.value, free.value


def _check(rc):
    if rc != 0:
        msg = load_library().cuacd_last_error().decode()
        if rc == -3:
            raise ScratchError(rc, msg)
        raise CuacdError(rc, msg)


def _int32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class GpuTree:
    """Lookahead tree search, hulls and Hausdorff distances on the GB300."""

    def __init__(self, **cfg):
        L = load_library()
        self.cfg = A.make_config(**cfg)
        err = C.c_int(0)
        self.h = L.cuacd_tree_create(C.byref(self.cfg), C.byref(err))
        if not self.h:
            raise CuacdError(err.value, L.cuacd_last_error().decode())
        self.plane_slots = L.cuacd_plane_slots(self.h)
        self.last_hull_fails = []

    def memory(self):
        """(device bytes held, {vertexCap, triCap, edgeCap, scratchWords})."""
        b, caps = C.c_uint64(), (C.c_uint64 * 4)()
        _check(load_library().cuacd_tree_memory(self.h, C.byref(b), caps))
        return b.value, dict(zip(("vertexCap", "triCap", "edgeCap", "scratchWords"), list(caps)))

    def schedule(self) -> dict:
        """The autotuner's state after the last run or hull batch."""
        out = (C.c_int32 * 4)()
        _check(load_library().cuacd_tree_schedule(self.h, out))
        return dict(warpMaxNv=out[0], bigJobNv=out[1], trial=bool(out[2]), tuned=out[3])

    def reserve_pools(self, vertexCap=0, triCap=0, edgeCap=0, scratchWords=0):
        """Grows the pools to at least these capacities (the configuration's
        units); never shrinks them."""
        caps = (C.c_uint64 * 4)(vertexCap, triCap, edgeCap, scratchWords)
        _check(load_library().cuacd_tree_reserve_pools(self.h, caps))

    def destroy(self):
        if getattr(self, "h", None):
            load_library().cuacd_tree_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    @property
    def vis_max(self):
        return 2048

    def set_profile(self, on: bool):
        load_library().cuacd_set_profile(self.h, int(on))

    @property
    def last_gpu_ms(self) -> float:
        """Device time of the last call (GpuTree.lastHullGpuMs, tree.ts:380)."""
        return float(load_library().cuacd_tree_last_gpu_ms(self.h))

    def kernel_bytes(self):
        """Algorithmic bytes of the last run's plan, emit and hull kernels."""
        b = (C.c_uint64 * 3)()
        _check(load_library().cuacd_tree_kernel_bytes(self.h, b))
        return [int(x) for x in b]

    KERNELS = ("reset", "plan", "scan", "emit", "hull", "record", "evaluate")

    def hd_stats(self) -> dict:
        """The last Hausdorff batch's tensor-core screen: exact distances,
        screened pairs and whether a tensor-core wait timed out."""
        b = (C.c_uint64 * 3)()
        _check(load_library().cuacd_tree_hd_stats(self.h, b))
        return dict(exact=int(b[0]), screened=int(b[1]), timeout=bool(b[2]))

    def kernel_ms(self) -> dict:
        """Per-kernel device time of the last profiled run (stats.kernelMs)."""
        ms = np.zeros(7, np.float32)
        _check(load_library().cuacd_tree_kernel_ms(self.h, A.fptr(ms)))
        return {k: float(v) for k, v in zip(self.KERNELS, ms)}

    # ---- GpuTree.run (tree.ts:449-661) ----
    def _args(self, seeds, edge_planes, depth, width, n_edge_cuts, refine):
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
        keep = [ma, ep]
        if refine:
            opts.refineRounds = refine["rounds"]
            opts.refineProbes = refine["probes"]
            sp = np.asarray(refine["spacing"], np.float32)
            keep.append(sp)
            opts.refineSpacing = A.fptr(sp)
        return ma, n, ep, opts, keep

    def run(self, seeds, edge_planes=None, depth=0, width=-1, n_edge_cuts=-1, refine=None):
        ma, n, ep, opts, keep = self._args(seeds, edge_planes, depth, width, n_edge_cuts, refine)
        out = (A.SeedResult * max(n, 1))()
        st = A.RunStats()
        _check(load_library().cuacd_tree_run(self.h, ma.arr, n, A.fptr(ep), self.plane_slots, C.byref(opts), out, C.byref(st)))
        return _result(out, st, n)

    def prepare(self, seeds, edge_planes=None, depth=0, width=-1, n_edge_cuts=-1, refine=None):
        """Upload seeds and planes once; launch() reruns the tree on them."""
        ma, n, ep, opts, keep = self._args(seeds, edge_planes, depth, width, n_edge_cuts, refine)
        _check(load_library().cuacd_tree_prepare(self.h, ma.arr, n, A.fptr(ep), self.plane_slots, C.byref(opts)))
        self._n = n

    def launch(self):
        _check(load_library().cuacd_tree_launch(self.h))

    def collect(self):
        n = self._n
        out = (A.SeedResult * max(n, 1))()
        st = A.RunStats()
        _check(load_library().cuacd_tree_collect(self.h, out, C.byref(st)))
        return _result(out, st, n)

    # ---- GpuTree.hullMeshes (tree.ts:382-443) ----
    def hull_meshes(self, meshes, hull_stage=0, no_export=False):
        meshes = [A.as_mesh(m) for m in meshes]
        n = len(meshes)
        if n == 0:
            return [], np.zeros(0, np.int32)
        ma = A.MeshArray(meshes)
        maxnv = max(m.nv for m in meshes)
        stride = 3 * 2 * min(self.cfg.hullMaxVerts, maxnv)
        tris = np.zeros(max(n * stride, 1), np.uint32)
        vol = np.zeros(n, np.float32)
        nt = np.zeros(n, np.uint32)
        status = np.zeros(n, np.int32)
        _check(load_library().cuacd_tree_hull_meshes(self.h, ma.arr, n, hull_stage, None if no_export else A.uptr(tris),
                                                     stride, A.fptr(vol), A.uptr(nt), _int32p(status)))
        out = []
        for i in range(n):
            if status[i] != 0:
                out.append(None)
            else:
                out.append(dict(tris=tris[i * stride: i * stride + 3 * nt[i]].reshape(-1, 3).copy(), volume=float(vol[i])))
        return out, status

    # ---- GpuTree.hullsWithHausdorff (tree.ts:671-756) ----
    def hulls_with_hausdorff(self, meshes):
        meshes = [A.as_mesh(m) for m in meshes]
        n = len(meshes)
        if n == 0:
            return []
        if n > HD_MAX_PAIRS:
            raise ValueError(f"hullsWithHausdorff: at most {HD_MAX_PAIRS} meshes per call")
        ma = A.MeshArray(meshes)
        maxnv = max(m.nv for m in meshes)
        stride = 3 * 2 * min(self.cfg.hullMaxVerts, maxnv)
        tris = np.zeros(max(n * stride, 1), np.uint32)
        vol = np.zeros(n, np.float32)
        nt = np.zeros(n, np.uint32)
        hd = np.zeros(n, np.float32)
        status = np.zeros(n, np.int32)
        _check(load_library().cuacd_tree_hulls_with_hausdorff(self.h, ma.arr, n, A.uptr(tris), stride, A.fptr(vol),
                                                              A.uptr(nt), A.fptr(hd), _int32p(status)))
        self.last_hull_fails = [int(s) for s in status]
        out = []
        for i in range(n):
            if status[i] != 0:
                out.append(None)
            else:
                out.append(dict(tris=tris[i * stride: i * stride + 3 * nt[i]].reshape(-1, 3).copy(), volume=float(vol[i]),
                                hausdorff=float(hd[i])))
        return out

    # ---- GpuTree.hausdorff (tree.ts:318-372) ----
    def hausdorff(self, pairs):
        n = len(pairs)
        if n == 0:
            return np.zeros(0, np.float32)
        if n > HD_MAX_PAIRS:
            raise ValueError(f"hausdorff: at most {HD_MAX_PAIRS} pairs per call")
        a = A.MeshArray([A.as_mesh(p[0]) for p in pairs])
        b = A.MeshArray([A.as_mesh(p[1]) for p in pairs])
        out = np.zeros(n, np.float32)
        _check(load_library().cuacd_tree_hausdorff(self.h, a.arr, b.arr, n, A.fptr(out)))
        return out

    # ---- debug readers (tree.ts:764-807) ----
    def plane_cuts(self, meshes, planes, mesh_of_cut=None, closed=False):
        """planeCut (src/cpu/cut.ts:33-315) on the GPU: cut k cuts
        meshes[mesh_of_cut[k]] (mesh k when None) by planes[k] = (a, b, c, d).
        Returns one (status, positive half, negative half) per cut; status 0
        or the cut's failure code (the halves are then None). The halves are
        the host cut's bit for bit. closed=True vouches that every mesh is
        closed (skips the open-edge search). The device time is
        last_cut_ms."""
        L = load_library()
        pl = np.ascontiguousarray(np.asarray(planes, np.float64).reshape(-1, 4))
        n = pl.shape[0]
        idx = np.arange(n, dtype=np.int32) if mesh_of_cut is None else np.ascontiguousarray(mesh_of_cut, np.int32)
        if idx.shape[0] != n:
            raise ValueError("one mesh index per plane")
        ma = A.MeshArray([A.as_mesh(m) for m in meshes])
        h = C.c_void_p()
        _check(L.cuacd_tree_plane_cuts(self.h, ma.arr, len(meshes), _int32p(idx),
                                       pl.ctypes.data_as(C.POINTER(C.c_double)), n, 1 if closed else 0, C.byref(h)))
        out = []
        try:
            self.last_cut_ms = float(L.cuacd_cuts_gpu_ms(h))
            for k in range(n):
                halves = []
                st = 0
                for side in (0, 1):
                    v = C.POINTER(C.c_float)()
                    t = C.POINTER(C.c_uint32)()
                    nv = C.c_uint32()
                    nt = C.c_uint32()
                    st = L.cuacd_cuts_half(h, k, side, C.byref(v), C.byref(nv), C.byref(t), C.byref(nt))
                    if st < 0:
                        _check(st)
                    if st != 0:
                        break
                    vv = np.ctypeslib.as_array(v, shape=(nv.value * 3,)).copy() if nv.value else np.zeros(0, np.float32)
                    tt = np.ctypeslib.as_array(t, shape=(nt.value * 3,)).copy() if nt.value else np.zeros(0, np.uint32)
                    halves.append(Mesh(vv.reshape(-1, 3), tt.reshape(-1, 3)))
                out.append((st, halves[0], halves[1]) if st == 0 else (st, None, None))
        finally:
            L.cuacd_cuts_free(h)
        return out

    def concave_planes(self, meshes, n_concave_edges=16, concave_eps=0.005, concave_threshold=3.49, seeds=None):
        """concaveEdgePlanes (src/cpu/concave.ts:25-92) of every mesh on the
        GPU: a list of (k, 4) float32 plane arrays (seeds[i] = mesh i's
        reservoir seed, 12345 when None)."""
        L = load_library()
        n = len(meshes)
        sd = np.full(n, 12345, np.uint32) if seeds is None else np.ascontiguousarray(np.asarray(seeds) & 0xFFFFFFFF,
                                                                                     np.uint32)
        ne = max(int(n_concave_edges), 0)
        out = np.zeros((max(n, 1), 4 * max(ne, 1), 4), np.float32)
        cnt = np.zeros(max(n, 1), np.int32)
        ma = A.MeshArray([A.as_mesh(m) for m in meshes])
        _check(L.cuacd_tree_concave_planes(self.h, ma.arr, n, ne, float(concave_eps), float(concave_threshold),
                                           A.uptr(sd), A.fptr(out), _int32p(cnt)))
        self.last_concave_ms = float(L.cuacd_tree_concave_ms(self.h))
        return [out[k, : cnt[k]].copy() for k in range(n)]

    def eval_cuts(self, mesh, planes):
        """The reference's CPU helpers per candidate plane, on the GPU: (n, 8)
        doubles per plane = split, |vol+|, |vol-|, hull+, hull-, rv+, rv-,
        max Hausdorff (cuacd_tree_eval_cuts). The device time is
        last_eval_ms."""
        L = load_library()
        pl = np.ascontiguousarray(np.asarray(planes, np.float64).reshape(-1, 4))
        out = np.zeros((pl.shape[0], 8), np.float64)
        ma = A.MeshArray([A.as_mesh(mesh)])
        _check(L.cuacd_tree_eval_cuts(self.h, ma.arr, pl.ctypes.data_as(C.POINTER(C.c_double)), pl.shape[0],
                                      out.ctypes.data_as(C.POINTER(C.c_double))))
        self.last_eval_ms = float(L.cuacd_tree_eval_cuts_ms(self.h))
        return out

    def items(self, first, n):
        w = np.zeros(20 * n, np.uint32)
        _check(load_library().cuacd_tree_read_items(self.h, first, n, A.uptr(w)))
        return w.reshape(n, 20)

    def parts(self, first, n):
        w = np.zeros(16 * n, np.uint32)
        _check(load_library().cuacd_tree_read_parts(self.h, first, n, A.uptr(w)))
        return w.reshape(n, 16)

    def jobs(self, first, n):
        w = np.zeros(24 * n, np.uint32)
        _check(load_library().cuacd_tree_read_jobs(self.h, first, n, A.uptr(w)))
        return w.reshape(n, 24)

    def part_geometry(self, idx):
        d = self.parts(idx, 1)[0]
        v = np.zeros(3 * d[1], np.float32)
        t = np.zeros(3 * d[3], np.uint32)
        e = np.zeros(8 * d[5], np.uint32)
        _check(load_library().cuacd_tree_read_part_geometry(self.h, idx, A.fptr(v), A.uptr(t), A.uptr(e)))
        return v.reshape(-1, 3), t.reshape(-1, 3), e.reshape(-1, 8)

    def read_part(self, idx):
        d = self.parts(idx, 1)[0]
        f = d.view(np.float32)
        v, t, e = self.part_geometry(idx)
        return dict(mesh=Mesh(v, t), edges=e, meshVol=float(f[6]), hullVol=float(f[7]), nPlanes=int(d[12]),
                    planeIds=[int(x) for x in d[8: 8 + d[12]]])

    def plane(self, idx):
        f = np.zeros(4, np.float32)
        _check(load_library().cuacd_tree_read_plane(self.h, idx, A.fptr(f)))
        return f

    read_plane = plane


def _result(out, st, n):
    seeds = []
    for i in range(n):
        s = out[i]
        seeds.append(dict(bestCut=s.bestCut, bestCost=s.bestCost if s.valid else float("inf"),
                          plane=list(s.plane) if s.valid else None))
    return dict(
        seeds=seeds, overflow=bool(st.overflow), hullFail=bool(st.hullFail), hullFailCount=st.hullFailCount,
        npOverflow=bool(st.npOverflow), pruned=st.pruned, jobsPerLevel=list(st.jobsPerLevel[: st.nLevels]),
        validJobs=st.validJobs, hullSlabWords=st.hullSlabWords, hullChunkSize=st.hullChunkSize, gpuMs=st.gpuMs,
    )


__all__ = ["GpuTree", "HD_MAX_PAIRS", "load_library", "library_path", "CuacdError", "ScratchError", "mesh_area"]
