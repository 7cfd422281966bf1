"""Table-by-table comparison of a CUDA GpuTree run with the CPU oracle's run
of the same inputs. Integer fields and geometry must be identical; volumes
and costs are float32 and must agree to a stated relative tolerance (they are
almost always bit-identical: both sides use the same float32 operation order
and exact hull volumes)."""
from __future__ import annotations

import numpy as np

VOL_RTOL = 1e-6   # meshVol / hullVol / level costs, relative
VOL_ATOL = 1e-9


def close(a, b, rtol=VOL_RTOL, atol=VOL_ATOL):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.all(np.abs(a - b) <= atol + rtol * np.maximum(np.abs(a), np.abs(b)))


def compare_level_tables(gpu, orc, res_g, res_o, n_seeds, geometry=True, label=""):
    """Jobs, child parts (with geometry) and items of every level."""
    jobs = res_g["jobsPerLevel"]
    assert jobs == res_o["jobsPerLevel"], (label, jobs, res_o["jobsPerLevel"])
    assert res_g["overflow"] == res_o["overflow"] and res_g["npOverflow"] == res_o["npOverflow"], label
    assert res_g["hullFailCount"] == res_o["hullFailCount"], (label, res_g["hullFailCount"], res_o["hullFailCount"])
    assert res_g["validJobs"] == res_o["validJobs"], (label, res_g["validJobs"], res_o["validJobs"])
    total = sum(jobs)
    if total == 0:
        return
    jg, jo = gpu.jobs(0, total), orc.jobs(0, total)
    # plane, parentItem, parentPart, valid, cutIdx, counts, offsets (the scratch
    # offset in off[6] comes from an atomic bump allocator and is not compared)
    mask = np.ones(24, bool)
    mask[22] = False
    bad = np.where((jg[:, mask] != jo[:, mask]).any(axis=1))[0]
    assert len(bad) == 0, (label, "jobs differ", bad[:5], jg[bad[:1]], jo[bad[:1]])
    nparts = n_seeds + 2 * total
    pg, po = gpu.parts(0, nparts), orc.parts(0, nparts)
    ints = [0, 1, 2, 3, 4, 5, 8, 9, 10, 11, 12, 13, 14, 15]
    bad = np.where((pg[:, ints] != po[:, ints]).any(axis=1))[0]
    assert len(bad) == 0, (label, "parts differ", bad[:5], pg[bad[:1]], po[bad[:1]])
    fg, fo = pg.view(np.float32), po.view(np.float32)
    assert close(fg[:, 6], fo[:, 6]), (label, "meshVol", np.abs(fg[:, 6] - fo[:, 6]).max())
    assert close(fg[:, 7], fo[:, 7]), (label, "hullVol", np.abs(fg[:, 7] - fo[:, 7]).max())
    nitems = n_seeds + total
    ig, io = gpu.items(0, nitems), orc.items(0, nitems)
    iints = [i for i in range(20) if i not in (12, 13, 14, 15)]
    bad = np.where((ig[:, iints] != io[:, iints]).any(axis=1))[0]
    assert len(bad) == 0, (label, "items differ", bad[:5], ig[bad[:1]], io[bad[:1]])
    assert close(ig[:, 12:16].view(np.float32), io[:, 12:16].view(np.float32)), (label, "level costs")
    if geometry:
        for p in range(nparts):
            if pg[p, 1] == 0 and pg[p, 3] == 0:
                continue
            vg, tg, eg = gpu.part_geometry(p)
            vo, to, eo = orc.part_geometry(p)
            assert np.array_equal(vg.view(np.uint32), vo.view(np.uint32)), (label, "verts", p)
            assert np.array_equal(tg, to), (label, "tris", p)
            assert np.array_equal(eg, eo), (label, "edges", p)


def compare_seeds(res_g, res_o, label="", gap_tol=1e-6):
    for k, (a, b) in enumerate(zip(res_g["seeds"], res_o["seeds"])):
        assert (a["plane"] is None) == (b["plane"] is None), (label, k)
        if a["plane"] is None:
            continue
        assert close([a["bestCost"]], [b["bestCost"]], rtol=1e-6, atol=1e-7), (label, k, a, b)
        if a["bestCut"] != b["bestCut"]:
            # only a near-tie may pick a different cut
            assert abs(a["bestCost"] - b["bestCost"]) <= gap_tol, (label, k, a, b)
        else:
            assert np.array_equal(np.float32(a["plane"]).view(np.uint32), np.float32(b["plane"]).view(np.uint32)), (label, k)
