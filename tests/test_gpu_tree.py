"""Parity of the CUDA lookahead tree with the CPU oracle, through the C ABI.

Every table of every level (jobs, child parts, items), the child geometry
(vertices, triangles, open edges), the chosen cuts and the run flags are
compared. Integers and geometry must be identical; volumes and costs agree to
1e-6 relative (parity.VOL_RTOL)."""
import importlib

import numpy as np
import pytest

import parity
import tree_cases
from fixtures import M, l_prism, square_torus, stairs

pytestmark = pytest.mark.gpu
gen = importlib.import_module("cuacd-web_gb300.meshgen")


@pytest.fixture(scope="module")
def GpuTree():
    return importlib.import_module("cuacd-web_gb300.tree").GpuTree


@pytest.mark.parametrize("case", tree_cases.ALL, ids=lambda c: c.__name__)
def test_reference_known_answers(GpuTree, case):
    case(GpuTree)


def run_both(GpuTree, oracle, seeds, planes=None, refine=None, run_depth=0, **cfg):
    g = GpuTree(**cfg)
    o = oracle.OracleTree(**cfg)
    rg = g.run(seeds, planes, depth=run_depth, refine=refine)
    ro = o.run(seeds, planes, depth=run_depth, refine=refine)
    return g, o, rg, ro


SMALL = dict(vertexCap=1 << 22, triCap=1 << 22, edgeCap=1 << 18, scratchWords=1 << 22, hullBudgetBytes=64 << 20,
             hullMaxVerts=1024)


def concave(oracle, m, n=16):
    return oracle.concave_planes(m, n)


CASES = {
    "cube_w3_d2": lambda o: ([M.unit_cube()], None, None, dict(width=3, width2=3, depth=2, nConcaveEdges=0, minEdgeDist=0.01)),
    "lshape_w9_d2": lambda o: ([M.normalize(M.l_shape())[0]], None, None, dict(width=9, width2=3, depth=2, nConcaveEdges=0)),
    "torus_w6_d3": lambda o: ([square_torus()], None, None, dict(width=6, width2=3, depth=3, nConcaveEdges=0)),
    "lprism_concave_d3_refine": lambda o: ([l_prism()], [concave(o, l_prism())],
                                           dict(rounds=2, probes=8, spacing=[0.1]),
                                           dict(width=6, width2=3, depth=3, nConcaveEdges=16)),
    "staircase8_config": lambda o: ([gen.staircase(8)], [concave(o, gen.staircase(8))],
                                    dict(rounds=2, probes=8, spacing=[0.05]),
                                    dict(width=6, width2=3, depth=3, nConcaveEdges=16, minEdgeDist=0.015)),
    "batch_mixed_seeds": lambda o: ([stairs(), square_torus(), gen.staircase(5), M.normalize(M.l_shape())[0]],
                                    [concave(o, stairs()), None, concave(o, gen.staircase(5)), None],
                                    dict(rounds=1, probes=5, spacing=[0.1, 0.1, 0.05, 0.0]),
                                    dict(width=6, width2=3, depth=2, nConcaveEdges=8)),
    "icosphere_random_planes": lambda o: ([gen.noisy_icosphere(2, seed=3)],
                                          [gen.random_planes(gen.noisy_icosphere(2, seed=3), 32, seed=1)], None,
                                          dict(width=6, width2=3, depth=2, nConcaveEdges=8)),
    "icosphere_L4_block_groups": lambda o: ([gen.noisy_icosphere(4, seed=0)], None, None,
                                            dict(width=3, width2=3, depth=2, nConcaveEdges=0)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_tree_tables_match_oracle(GpuTree, oracle, name):
    seeds, planes, refine, cfg = CASES[name](oracle)
    cfg = {**SMALL, **cfg}
    g, o, rg, ro = run_both(GpuTree, oracle, seeds, planes, refine, **cfg)
    assert not rg["overflow"]
    parity.compare_level_tables(g, o, rg, ro, len(seeds), label=name)
    parity.compare_seeds(rg, ro, label=name)


def test_resident_relaunch_is_identical(GpuTree, oracle):
    seeds = [gen.staircase(8), stairs()]
    planes = [concave(oracle, s) for s in seeds]
    cfg = {**SMALL, **dict(width=6, width2=3, depth=3, nConcaveEdges=16)}
    g = GpuTree(**cfg)
    refine = dict(rounds=2, probes=8, spacing=[0.05, 0.1])
    r0 = g.run(seeds, planes, refine=refine)
    g.prepare(seeds, planes, refine=refine)
    for _ in range(3):
        g.launch()
    r1 = g.collect()
    assert r0["seeds"] == r1["seeds"]
    assert r0["validJobs"] == r1["validJobs"]


def test_empty_and_pool_overflow(GpuTree, oracle):
    g = GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0, **SMALL)
    r = g.run([])
    assert r["seeds"] == [] and not r["overflow"]
    # tiny vertex pool: the run reports overflow (a flag, not an error)
    cfg = dict(width=6, width2=3, depth=2, nConcaveEdges=0, vertexCap=3000, triCap=1 << 16, edgeCap=1 << 14,
               scratchWords=1 << 16, hullBudgetBytes=16 << 20, hullMaxVerts=256)
    seed = gen.noisy_icosphere(3)
    rg = GpuTree(**cfg).run([seed])
    ro = oracle.OracleTree(**cfg).run([seed])
    assert rg["overflow"] and ro["overflow"]


def test_reserved_pools_end_the_overflow(GpuTree, oracle):
    """cuacd_tree_reserve_pools: the run that overflowed the small pools
    fits once they grow, equals the run on pools of that size from the
    start, and the handle's device bytes grow by the pools' growth."""
    cfg = dict(width=6, width2=3, depth=2, nConcaveEdges=0, vertexCap=3000, triCap=1 << 16, edgeCap=1 << 14,
               scratchWords=1 << 16, hullBudgetBytes=16 << 20, hullMaxVerts=256)
    seed = gen.noisy_icosphere(3)
    g = GpuTree(**cfg)
    assert g.run([seed])["overflow"]
    b0, c0 = g.memory()
    big = dict(vertexCap=1 << 20, triCap=1 << 20, edgeCap=1 << 15, scratchWords=1 << 17)
    g.reserve_pools(**big)
    b1, c1 = g.memory()
    assert c1 == big
    unit = dict(vertexCap=4, triCap=4, edgeCap=32, scratchWords=4)
    assert b1 - b0 == sum(unit[k] * (c1[k] - c0[k]) for k in unit)
    g.reserve_pools(vertexCap=1000, triCap=1000)  # pools never shrink
    assert g.memory()[1] == big
    r = g.run([seed])
    ref = GpuTree(**dict(cfg, **big)).run([seed])
    assert not r["overflow"] and r["seeds"] == ref["seeds"] and r["validJobs"] == ref["validJobs"]


def test_autotuned_schedules_match_oracle(GpuTree, oracle):
    """The autotuner tries each schedule (warp/block thresholds of the hull
    and of plan/emit) on the first runs of a part-size distribution, then
    keeps the fastest. Seeds of 642, ~3,000 and 50 points put parts on both
    sides of every threshold; every run's tables equal the oracle's."""
    seeds = [gen.noisy_icosphere(3, seed=1), M.normalize(gen.blob_mesh(10, 36, seed=3))[0], gen.staircase(8)]
    assert 2048 < seeds[1].nv <= 4096
    cfg = {**SMALL, **dict(width=3, width2=3, depth=2, nConcaveEdges=0, hullMaxVerts=4096)}
    g = GpuTree(**cfg)
    o = oracle.OracleTree(**cfg)
    ro = o.run(seeds)
    seen = []
    for k in range(6):
        rg = g.run(seeds)
        seen.append(g.schedule())
        assert not rg["overflow"]
        parity.compare_level_tables(g, o, rg, ro, len(seeds), label=f"run {k}")
        parity.compare_seeds(rg, ro, label=f"run {k}")
    assert [s["trial"] for s in seen] == [True] * 4 + [False] * 2
    assert {(s["warpMaxNv"], s["bigJobNv"]) for s in seen[:4]} == {(1024, 2048), (512, 2048), (256, 2048),
                                                                      (1024, 4096)}
    assert seen[4] == seen[5] and seen[5]["tuned"] >= 1
    # a fixed warpMaxNv turns the tuner off
    g2 = GpuTree(**{**cfg, "warpMaxNv": 512})
    g2.run(seeds)
    assert g2.schedule() == dict(warpMaxNv=512, bigJobNv=2048, trial=False, tuned=0)


def test_invalid_config_raises(GpuTree):
    with pytest.raises(Exception):
        GpuTree(width=4)
    with pytest.raises(Exception):
        GpuTree(depth=5)
