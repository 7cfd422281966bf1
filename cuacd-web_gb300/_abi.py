"""ctypes mirrors of the C structs in include/cuacd.h."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .mesh import Mesh

NONE = 0xFFFFFFFF


class TreeConfig(C.Structure):
    """cuacd_tree_config — the reference's TreeConfig (src/gpu/tree.ts:14-46)."""

    _fields_ = [
        ("width", C.c_int32),
        ("width2", C.c_int32),
        ("depth", C.c_int32),
        ("nConcaveEdges", C.c_int32),
        ("minEdgeDist", C.c_float),
        ("hullMaxVerts", C.c_int32),
        ("vertexCap", C.c_uint64),
        ("triCap", C.c_uint64),
        ("edgeCap", C.c_uint64),
        ("scratchWords", C.c_uint64),
        ("hullBudgetBytes", C.c_uint64),
        ("pruneLastLevel", C.c_int32),
        ("warpMaxNv", C.c_int32),
        ("hdScreenMinTris", C.c_int32),
        ("autotune", C.c_int32),
    ]


class MeshRef(C.Structure):
    """cuacd_mesh — borrowed pointers to one mesh's arrays."""

    _fields_ = [
        ("verts", C.POINTER(C.c_float)),
        ("tris", C.POINTER(C.c_uint32)),
        ("nv", C.c_uint32),
        ("nt", C.c_uint32),
    ]


class RunOpts(C.Structure):
    """cuacd_run_opts — GpuTree.run's opts (tree.ts:449-453)."""

    _fields_ = [
        ("depth", C.c_int32),
        ("width", C.c_int32),
        ("nEdgeCuts", C.c_int32),
        ("refineRounds", C.c_int32),
        ("refineProbes", C.c_int32),
        ("reserved", C.c_int32),
        ("refineSpacing", C.POINTER(C.c_float)),
    ]


class SeedResult(C.Structure):
    """cuacd_seed_result — SeedResult (tree.ts:69-73)."""

    _fields_ = [
        ("bestCut", C.c_int32),
        ("bestCost", C.c_float),
        ("plane", C.c_float * 4),
        ("valid", C.c_int32),
        ("reserved", C.c_int32),
    ]


class RunStats(C.Structure):
    """cuacd_run_stats — TreeRunResult flags and stats (tree.ts:75-85)."""

    _fields_ = [
        ("overflow", C.c_uint32),
        ("hullFail", C.c_uint32),
        ("hullFailCount", C.c_uint32),
        ("npOverflow", C.c_uint32),
        ("pruned", C.c_uint32),
        ("nLevels", C.c_uint32),
        ("jobsPerLevel", C.c_uint32 * 4),
        ("validJobs", C.c_uint64),
        ("hullSlabWords", C.c_uint32),
        ("hullChunkSize", C.c_uint32),
        ("gpuMs", C.c_float),
        ("reserved", C.c_uint32),
    ]


# DEFAULT_TREE_CONFIG (tree.ts:33-46). The reference lists width2 5, which its
# own constructor rejects (not a multiple of 3); every caller passes 3
# (decompose.ts:91), so 3 is the default here.
DEFAULT_TREE_CONFIG = dict(
    width=60,
    width2=3,
    depth=2,
    nConcaveEdges=32,
    minEdgeDist=0.0125,
    hullMaxVerts=4096,
    vertexCap=64 << 20,
    triCap=64 << 20,
    edgeCap=1 << 20,
    scratchWords=48 << 20,
    hullBudgetBytes=256 << 20,
    pruneLastLevel=1,
    warpMaxNv=0,
    hdScreenMinTris=0,
    autotune=1,
)


def make_config(**kw) -> TreeConfig:
    d = dict(DEFAULT_TREE_CONFIG)
    for k, v in kw.items():
        if k not in d:
            raise KeyError(f"unknown tree config field {k!r}")
        d[k] = v
    c = TreeConfig()
    for k, v in d.items():
        setattr(c, k, int(v) if k != "minEdgeDist" else float(v))
    return c


class MeshArray:
    """Keeps numpy arrays alive while a C array of cuacd_mesh points at them."""

    def __init__(self, meshes):
        self.keep = []
        self.arr = (MeshRef * max(1, len(meshes)))()
        for i, m in enumerate(meshes):
            v = np.ascontiguousarray(m.verts, dtype=np.float32)
            t = np.ascontiguousarray(m.tris, dtype=np.uint32)
            self.keep += [v, t]
            self.arr[i].verts = v.ctypes.data_as(C.POINTER(C.c_float))
            self.arr[i].tris = t.ctypes.data_as(C.POINTER(C.c_uint32))
            self.arr[i].nv = v.shape[0]
            self.arr[i].nt = t.shape[0]
        self.n = len(meshes)


def fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def uptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def item_view(w: np.ndarray) -> dict:
    """ItemView of a 20-word item record (tree.ts:48-58, 621-629)."""
    f = w.view(np.float32)
    return dict(
        partIds=w[0:8].copy(), np=int(w[8]), srcPart=int(w[9]), initialCut=int(w[10]), nLevels=int(w[11]),
        levelCosts=f[12:16].copy(), flags=int(w[16]), parentItem=int(w[17]), cutIdx=int(w[18]),
    )


def as_mesh(x) -> Mesh:
    return x if isinstance(x, Mesh) else Mesh(*x)


class DecomposeOpts(C.Structure):
    """cuacd_decompose_opts — DecomposeOptions (decompose.ts:26-78)."""

    _fields_ = [
        ("threshold", C.c_float),
        ("maxIters", C.c_int32),
        ("width", C.c_int32),
        ("width2", C.c_int32),
        ("depth", C.c_int32),
        ("maxNCutting", C.c_int32),
        ("nConcaveEdges", C.c_int32),
        ("concaveEps", C.c_float),
        ("concaveThreshold", C.c_float),
        ("concaveIters", C.c_int32),
        ("normalize", C.c_int32),
        ("requireClosed", C.c_int32),
        ("validateCuts", C.c_int32),
        ("refineRounds", C.c_int32),
        ("refineProbes", C.c_int32),
        ("mergeHulls", C.c_int32),
        ("mergeRounds", C.c_int32),
        ("mergePlaneTol", C.c_float),
        ("profile", C.c_int32),
        ("threads", C.c_int32),
        ("verbose", C.c_int32),
        ("streams", C.c_int32),
        ("tree", TreeConfig),
    ]


class PartView(C.Structure):
    """cuacd_part_view — one Part (part.ts:9-22) of a result."""

    _fields_ = [
        ("verts", C.POINTER(C.c_float)),
        ("tris", C.POINTER(C.c_uint32)),
        ("hullVerts", C.POINTER(C.c_float)),
        ("hullTris", C.POINTER(C.c_uint32)),
        ("seams", C.POINTER(C.c_double)),
        ("nv", C.c_uint32),
        ("nt", C.c_uint32),
        ("hullNv", C.c_uint32),
        ("hullNt", C.c_uint32),
        ("nSeams", C.c_uint32),
        ("stuck", C.c_int32),
        ("stuckReason", C.c_int32),
        ("merged", C.c_int32),
        ("meshVol", C.c_double),
        ("hullVol", C.c_double),
        ("hausdorff", C.c_double),
    ]


class DecomposeStats(C.Structure):
    """cuacd_decompose_stats — DecomposeResult.stats + MergeStats."""

    _fields_ = [
        ("iterations", C.c_int32),
        ("treeRuns", C.c_int32),
        ("hullFailRuns", C.c_int32),
        ("nParts", C.c_int32),
        ("mergeRounds", C.c_int32),
        ("merges", C.c_int32),
        ("pairsHulled", C.c_int32),
        ("pairsHausdorff", C.c_int32),
        ("candidates", C.c_uint64),
        ("totalMs", C.c_double),
        ("treeMs", C.c_double),
        ("cutMs", C.c_double),
        ("concaveMs", C.c_double),
        ("hullMs", C.c_double),
        ("hausdorffMs", C.c_double),
        ("mergeMs", C.c_double),
        ("gpuMs", C.c_double),
    ]


class PartIn(C.Structure):
    """cuacd_part_in — a part handed to the merge pass (part.ts:9-22)."""

    _fields_ = [
        ("mesh", MeshRef),
        ("hull", MeshRef),
        ("meshVol", C.c_double),
        ("hullVol", C.c_double),
        ("hausdorff", C.c_double),
        ("seams", C.POINTER(C.c_double)),
        ("nSeams", C.c_uint32),
        ("merged", C.c_int32),
    ]


class MergeOpts(C.Structure):
    """cuacd_merge_opts — MergeOptions (merge.ts:25-42)."""

    _fields_ = [
        ("threshold", C.c_float),
        ("maxRounds", C.c_int32),
        ("planeTol", C.c_double),
        ("hullEps", C.c_double),
        ("verbose", C.c_int32),
        ("reserved", C.c_int32),
    ]


class ServerStats(C.Structure):
    """cuacd_server_state — device memory and queue of a server."""

    _fields_ = [
        ("budgetBytes", C.c_uint64),
        ("deviceBytes", C.c_uint64),
        ("peakDeviceBytes", C.c_uint64),
        ("workingSetBytes", C.c_uint64),
        ("projectedBytes", C.c_uint64),
        ("admitted", C.c_uint64),
        ("rejected", C.c_uint64),
        ("queued", C.c_int32),
        ("active", C.c_int32),
    ]


class MergeStats(C.Structure):
    """cuacd_merge_stats — MergeStats (merge.ts:54-66)."""

    _fields_ = [
        ("rounds", C.c_int32),
        ("merges", C.c_int32),
        ("pairsHulled", C.c_int32),
        ("pairsHausdorff", C.c_int32),
        ("hullFallbacks", C.c_int32),
        ("reserved", C.c_int32),
        ("hullMs", C.c_double),
        ("hausdorffMs", C.c_double),
        ("totalMs", C.c_double),
    ]


class PartArray:
    """Keeps numpy arrays alive while a C array of cuacd_part_in points at them."""

    def __init__(self, parts):
        self.keep = []
        self.arr = (PartIn * max(1, len(parts)))()
        for i, p in enumerate(parts):
            for name in ("mesh", "hull"):
                m = getattr(p, name)
                v = np.ascontiguousarray(m.verts, dtype=np.float32)
                t = np.ascontiguousarray(m.tris, dtype=np.uint32)
                self.keep += [v, t]
                ref = getattr(self.arr[i], name)
                ref.verts = v.ctypes.data_as(C.POINTER(C.c_float))
                ref.tris = t.ctypes.data_as(C.POINTER(C.c_uint32))
                ref.nv = v.shape[0]
                ref.nt = t.shape[0]
            s = np.ascontiguousarray(np.asarray(getattr(p, "seams", []) or [], np.float64).reshape(-1, 4))
            self.keep.append(s)
            self.arr[i].seams = s.ctypes.data_as(C.POINTER(C.c_double))
            self.arr[i].nSeams = s.shape[0]
            self.arr[i].meshVol = float(p.meshVol)
            self.arr[i].hullVol = float(p.hullVol)
            hd = getattr(p, "hausdorff", None)
            self.arr[i].hausdorff = float("nan") if hd is None else float(hd)
            self.arr[i].merged = int(getattr(p, "merged", 1) or 1)
        self.n = len(parts)
