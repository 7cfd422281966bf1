"""decompose(mesh, options) end to end on the GPU: the reference's known
answers (tests/decompose.test.ts:10-53, tests/merge.test.ts:76-97) and the
batched form against one mesh at a time (same parts, bit for bit)."""
import numpy as np
import pytest

from conftest import pkg
from fixtures import M, square_torus, stairs

D = pkg("decompose")
G = pkg("meshgen")
T = pkg("tree")
P = pkg("part")

# smallTree (tests/decompose.test.ts:8)
SMALL_TREE = dict(vertexCap=4 << 20, triCap=4 << 20, edgeCap=1 << 18, scratchWords=4 << 20, hullBudgetBytes=32 << 20,
                  hullMaxVerts=1024)

pytestmark = pytest.mark.gpu


def _cost(p):
    return P.part_cost(p.meshVol, p.hullVol, p.hausdorff)


def _check_parts(r, vol, thr):
    total = 0.0
    for p in r.parts:
        assert M.is_closed(p.mesh)
        assert _cost(p) < thr + 1e-6 or p.stuck, _cost(p)
        total += M.volume(p.mesh)
    assert abs(total - vol) < 1e-4, total


def test_cube_stays_one_part():
    r = D.decompose(M.unit_cube(), maxIters=5, threshold=0.05, tree=SMALL_TREE)
    assert len(r.parts) == 1
    assert abs(M.volume(r.parts[0].mesh) - 1) < 1e-6
    assert r.iterations == 1


def test_l_shape_two_parts():
    r = D.decompose(M.l_shape(), maxIters=50, threshold=0.05, width=30, tree=SMALL_TREE, mergeHulls=False)
    assert 2 <= len(r.parts) <= 10, len(r.parts)
    _check_parts(r, 1.5, 0.05)
    # with the merge pass the L ends at exactly 2 parts (merge.test.ts:89-97)
    r = D.decompose(M.l_shape(), maxIters=50, threshold=0.05, width=30, tree=SMALL_TREE, mergeHulls=True)
    assert len(r.parts) == 2, len(r.parts)
    _check_parts(r, 1.5, 0.05)


def test_stairs_and_torus():
    r = D.decompose(stairs(), maxIters=50, threshold=0.05, width=30, tree=SMALL_TREE)
    assert 3 <= len(r.parts) <= 6, len(r.parts)
    _check_parts(r, 6.0, 0.05)
    r = D.decompose(square_torus(), maxIters=50, threshold=0.05, width=30, tree=SMALL_TREE)
    assert len(r.parts) >= 4, len(r.parts)
    _check_parts(r, 1.5, 0.05)


def _same(ra, rb):
    assert len(ra.parts) == len(rb.parts)
    assert ra.iterations == rb.iterations
    for a, b in zip(ra.parts, rb.parts):
        assert np.array_equal(a.mesh.verts, b.mesh.verts) and np.array_equal(a.mesh.tris, b.mesh.tris)
        assert np.array_equal(a.hull.verts, b.hull.verts) and np.array_equal(a.hull.tris, b.hull.tris)
        assert a.meshVol == b.meshVol and a.hullVol == b.hullVol and a.hausdorff == b.hausdorff
        assert a.stuck == b.stuck and a.merged == b.merged and a.seams == b.seams


def test_batched_equals_one_at_a_time():
    meshes = [M.l_shape(), stairs(), square_torus(), M.unit_cube(), G.staircase(6)]
    opts = dict(maxIters=20, threshold=0.05, width=6, depth=2, tree=SMALL_TREE)
    d = D.Decomposer(**opts)
    try:
        batched = d.decompose_many(meshes, batched=True)
        plain = d.decompose_many(meshes, batched=False)
        alone = [d.decompose(m) for m in meshes]
    finally:
        d.destroy()
    for b, p, a in zip(batched, plain, alone):
        _same(b, p)
        _same(b, a)
    # the batch split over three engines (streams), each on its own host
    # thread and CUDA stream: the same parts
    d = D.Decomposer(**opts, streams=3)
    try:
        grouped = d.decompose_many(meshes, batched=True)
    finally:
        d.destroy()
    for g, a in zip(grouped, alone):
        _same(g, a)


def test_server_same_alone_and_in_the_mix():
    """Continuous batching: requests arrive while others run, with two
    thresholds; every result equals the mesh decomposed alone, and the
    admission's projection of device memory is never below what the trees
    hold."""
    opts = dict(maxIters=20, threshold=0.05, width=6, depth=2, tree=SMALL_TREE)
    meshes = [M.l_shape(), stairs(), square_torus(), G.staircase(6), G.noisy_icosphere(2, seed=4), M.unit_cube()]
    thresholds = [0.05, 0.1, 0.05, 0.1, 0.05, 0.05]
    s = D.Server(**opts)
    try:
        tickets = {}
        arrivals = {0: [0, 1], 1: [2], 2: [3, 4], 4: [5]}
        step, most_active = 0, 0
        while step < 200 and (len(tickets) < len(meshes) or s.pending):
            for k in arrivals.get(step, []):
                tickets[k] = s.submit(meshes[k], thresholds[k])
            s.step()
            st = s.stats()
            most_active = max(most_active, st["active"])
            assert st["projectedBytes"] >= st["deviceBytes"], st
            step += 1
        got = {k: s.take(t) for k, t in tickets.items()}
        st = s.stats()
    finally:
        s.destroy()
    assert st["admitted"] == len(meshes) and st["rejected"] == 0 and most_active >= 3
    assert st["peakDeviceBytes"] <= st["budgetBytes"]
    assert all(r is not None for r in got.values())
    for k, m in enumerate(meshes):
        alone = D.decompose(m, **dict(opts, threshold=thresholds[k]))
        _same(got[k], alone)
        assert got[k].stats["totalMs"] > 0


def test_server_admits_by_device_memory():
    """Two meshes whose pools must grow: with a budget between the projected
    bytes of the first alone and of both, the second waits in the queue
    until the first finishes, and the trees never hold more than the
    budget; both results equal the meshes decomposed alone."""
    tree = dict(SMALL_TREE, vertexCap=1 << 16, triCap=1 << 16)
    opts = dict(maxIters=20, threshold=0.05, width=6, depth=2, tree=tree)
    a, b = G.noisy_icosphere(3, seed=1), G.noisy_icosphere(3, seed=2)

    def run(budget):
        s = D.Server(admit_bytes=budget, **opts)
        try:
            ta = s.submit(a)
            s.step()
            p1 = s.stats()["projectedBytes"]
            tb = s.submit(b)
            s.step()
            st = s.stats()
            p2, queued, most_active = st["projectedBytes"], st["queued"], st["active"]
            n = 0
            while s.pending and n < 100:
                s.step()
                st = s.stats()
                most_active = max(most_active, st["active"])
                assert st["deviceBytes"] <= st["projectedBytes"] <= budget or st["active"] <= 1, st
                n += 1
            return p1, p2, queued, most_active, s.take(ta), s.take(tb), s.stats()
        finally:
            s.destroy()

    p1, p2, queued, most_active, _, _, _ = run(1 << 40)
    assert queued == 0 and most_active == 2 and p2 > p1
    budget = (p1 + p2) // 2
    _, _, queued, most_active, ra, rb, st = run(budget)
    print(f"admission: one request {p1} bytes projected, two {p2}; budget {budget}, peak held "
          f"{st['peakDeviceBytes']}")
    assert queued == 1 and most_active == 1 and st["peakDeviceBytes"] <= budget
    # alone on pools large enough from the start (the parts do not depend on
    # the pools' sizes)
    _same(ra, D.decompose(a, **dict(opts, tree=SMALL_TREE)))
    _same(rb, D.decompose(b, **dict(opts, tree=SMALL_TREE)))


def test_server_slots_queue_bound_and_oversize_requests():
    opts = dict(maxIters=20, threshold=0.05, width=6, depth=2, tree=SMALL_TREE)
    s = D.Server(max_active=1, max_queue=2, **opts)
    try:
        st = s.stats()
        total, _ = T.device_memory()
        assert st["budgetBytes"] == total // 5 * 4 and st["deviceBytes"] > 0
        t = [s.submit(M.l_shape()), s.submit(stairs())]
        with pytest.raises(T.CuacdError) as e:
            s.submit(M.unit_cube())
        assert e.value.code == D.Server.E_BUSY
        assert s.stats()["rejected"] == 1 and s.stats()["queued"] == 2
        s.step()  # one slot: one runs, one waits, and the queue has room again
        st = s.stats()
        assert st["active"] <= 1 and st["queued"] <= 1
        t.append(s.submit(M.unit_cube()))
        n = 0
        while s.pending and n < 200:
            s.step()
            assert s.stats()["active"] <= 1
            n += 1
        assert all(s.take(x) is not None for x in t)
    finally:
        s.destroy()
    # a mesh whose working set alone exceeds the budget is refused at once
    s = D.Server(admit_bytes=1 << 20, **opts)
    try:
        with pytest.raises(T.CuacdError) as e:
            s.submit(G.noisy_icosphere(3, seed=1))
        assert e.value.code == -2 and "working set" in str(e.value)
    finally:
        s.destroy()


def test_staircase_configuration():
    # the staircase decomposition's settings: threshold 0.1, width 6,
    # width2 3, depth 3, maxNCutting 160, 16 concave edges, 2 refinement
    # rounds, merging on
    m = G.staircase(8)
    r = D.decompose(m, threshold=0.1, width=6, width2=3, depth=3, maxNCutting=160, nConcaveEdges=16, refineRounds=2,
                    mergeHulls=True)
    assert len(r.parts) >= 2
    _check_parts(r, M.volume(m), 0.1)
    assert r.stats["candidates"] > 0 and r.stats["treeRuns"] >= 1


def _hull_issues(h, pts):
    # hull_output.test.ts:13-38: closed, outward, no degenerate face, every
    # point of the part inside within 1e-4 of its extent
    V = h.verts.astype(np.float64)
    T = h.tris
    if not M.is_closed(h):
        return "not closed"
    if not M.signed_volume(h) > 0:
        return "not outward"
    P = pts.verts.astype(np.float64)
    ext = P.max() - P.min()
    bad, max_out = 0, 0.0
    for a, b, c in T:
        u, w = V[b] - V[a], V[c] - V[a]
        n = np.cross(u, w)
        l = np.linalg.norm(n)
        if not l > 1e-6 * np.linalg.norm(u) * np.linalg.norm(w):
            bad += 1
            continue
        n /= l
        max_out = max(max_out, float((P @ n - n @ V[a]).max()))
    if bad:
        return f"{bad} degenerate faces"
    if max_out > 1e-4 * ext:
        return f"points outside by {max_out / ext:.2e} of the extent"
    return None


@pytest.mark.parametrize("merge", [False, True])
def test_output_hulls_are_clean(merge):
    # every output hull (cleaned by cleanHullFaces) is a clean closed convex
    # mesh around its part, with and without merging (hull_output.test.ts)
    for name, m in (("stairs", stairs()), ("blob", G.blob_mesh(6, 28, 5))):
        r = D.decompose(m, maxIters=100, threshold=0.05, mergeHulls=merge, tree=dict(SMALL_TREE, hullMaxVerts=4096))
        bad = [(i, _hull_issues(p.hull, p.mesh)) for i, p in enumerate(r.parts)]
        bad = [b for b in bad if b[1]]
        assert not bad, (name, merge, len(r.parts), bad[:5])
