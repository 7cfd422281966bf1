"""The server's working-set estimate (cuacd_pool_working_set) against the
oracle's tree: a lookahead run with the estimate's pools (vertex, triangle,
open-edge and scratch) does not overflow, with concave planes and two
refinement rounds, at depth 2 and 3. CPU only (the oracle's tree)."""
import ctypes as C

import pytest

from conftest import pkg

A = pkg("_abi")
G = pkg("meshgen")
M = pkg("mesh")
T = pkg("tree")


def estimate(cfg, mesh):
    L = T.load_library()
    L.cuacd_pool_working_set.argtypes = [C.POINTER(A.TreeConfig), C.c_uint32, C.c_uint32, C.POINTER(C.c_uint64)]
    caps = (C.c_uint64 * 4)()
    c = A.make_config(**cfg)
    assert L.cuacd_pool_working_set(C.byref(c), mesh.nv, mesh.nt, caps) == 0
    return dict(zip(("vertexCap", "triCap", "edgeCap", "scratchWords"), list(caps)))


MESHES = {
    "staircase8": lambda: G.staircase(8),
    "icosphere2": lambda: G.noisy_icosphere(2, seed=4),
    "icosphere3": lambda: G.noisy_icosphere(3, seed=1),
    "blob": lambda: G.blob_mesh(6, 26, seed=3),
}


@pytest.mark.parametrize("depth", [2, 3])
@pytest.mark.parametrize("name", sorted(MESHES))
def test_estimate_holds_one_run(oracle, name, depth):
    mesh = M.normalize(MESHES[name]())[0]
    cfg = dict(width=6, width2=3, depth=depth, nConcaveEdges=16, hullBudgetBytes=32 << 20, hullMaxVerts=4096)
    caps = estimate(cfg, mesh)
    planes = oracle.concave_planes(mesh, 16)
    t = oracle.OracleTree(**cfg, **caps)
    r = t.run([mesh], [planes], refine=dict(rounds=2, probes=8, spacing=[0.05]))
    assert not r["overflow"] and not r["npOverflow"], (name, depth, caps)
    # and the estimate is not a blanket: the vertex pool at a fifth of it overflows
    small = dict(caps, vertexCap=caps["vertexCap"] // 5)
    r2 = oracle.OracleTree(**cfg, **small).run([mesh], [planes], refine=dict(rounds=2, probes=8, spacing=[0.05]))
    assert r2["overflow"], (name, depth, caps)
