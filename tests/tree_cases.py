"""Known-answer cases of the reference's GPU tree tests
(tests/gpu_tree.test.ts:8-108), written against the GpuTree interface so the
same cases check the CPU oracle and the CUDA engine."""
from __future__ import annotations

import numpy as np

from fixtures import M

SMALL = dict(vertexCap=1 << 20, triCap=1 << 20, edgeCap=1 << 16, scratchWords=1 << 20, hullBudgetBytes=8 << 20,
             hullMaxVerts=256)


def part_vols(tree, idx):
    d = tree.parts(idx, 1)[0]
    f = d.view(np.float32)
    return float(f[6]), float(f[7]), int(d[12])


def cube_depth1(make):
    tree = make(width=3, width2=3, depth=2, nConcaveEdges=0, minEdgeDist=0.01, **SMALL)
    res = tree.run([M.unit_cube()], depth=1)
    assert not res["overflow"] and not res["hullFail"]
    assert res["jobsPerLevel"][0] == 3 + tree.plane_slots
    items = tree.items(1, 3)
    for j in range(3):
        it = items[j]
        assert it[16] == 1 and it[8] == 2
        for p in range(2):
            mv, hv, npl = part_vols(tree, int(it[p]))
            assert abs(mv - 0.5) < 1e-5 and abs(hv - 0.5) < 1e-4 and npl == 1
        assert abs(it[12:16].view(np.float32)[0]) < 1e-4
    assert abs(res["seeds"][0]["bestCost"]) < 1e-4
    return tree, res


def cube_depth2(make):
    tree = make(width=3, width2=3, depth=2, nConcaveEdges=0, minEdgeDist=0.01, **SMALL)
    res = tree.run([M.unit_cube()], depth=2)
    assert not res["overflow"] and not res["hullFail"]
    assert res["jobsPerLevel"][1] == (3 + tree.plane_slots) * 3
    base = 1 + res["jobsPerLevel"][0]
    items = tree.items(base, 9)
    checked = 0
    for j in range(9):
        it = items[j]
        assert it[16] == 1 and it[8] == 3, (j, it)
        vols = []
        for p in range(3):
            mv, hv, _ = part_vols(tree, int(it[p]))
            vols.append(mv)
            assert abs(hv - mv) < 2e-4
            checked += 1
        vols.sort()
        assert abs(vols[0] - 0.25) < 1e-5 and abs(vols[1] - 0.25) < 1e-5 and abs(vols[2] - 0.5) < 1e-5
    assert checked == 27
    return tree, res


def l_shape_best(make):
    tree = make(width=9, width2=3, depth=2, nConcaveEdges=0, minEdgeDist=0.0125, **SMALL)
    mesh, _, _ = M.normalize(M.l_shape())
    res = tree.run([mesh], depth=2)
    assert not res["overflow"] and not res["hullFail"]
    s = res["seeds"][0]
    pl = s["plane"]
    assert pl is not None
    is_x = abs(pl[0] - 1) < 1e-6 and abs(pl[3]) < 1e-3
    is_z = abs(pl[2] - 1) < 1e-6 and abs(pl[3]) < 1e-3
    assert is_x or is_z, pl
    assert abs(s["bestCost"]) < 1e-3
    return tree, res


def off_center_box(make):
    tree = make(width=6, width2=3, depth=2, nConcaveEdges=0, minEdgeDist=0.01, **SMALL)
    box = M.make_box((0.2, -0.7, 0.1), (0.9, 0.3, 0.8))
    total = M.volume(box)
    res = tree.run([box], depth=2)
    n0, n1 = res["jobsPerLevel"][0], res["jobsPerLevel"][1]
    for first, n in ((1, n0), (1 + n0, n1)):
        for it in tree.items(first, n):
            if it[16] != 1:
                continue
            s = 0.0
            for p in range(it[8]):
                mv, hv, _ = part_vols(tree, int(it[p]))
                assert abs(hv - mv) < 1e-4
                s += mv
            assert abs(s - total) < 1e-5
    return tree, res


ALL = [cube_depth1, cube_depth2, l_shape_best, off_center_box]
