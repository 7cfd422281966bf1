"""seamPlane and filteredConcat of the merge pass (src/merge.ts:114-157) in the
library (csrc/decompose.cpp, through cuacd_seam_plane / cuacd_filtered_concat)
against the oracle's restatement (oracle/merge_oracle.cpp): the same plane
bit for bit (or none), the same kept triangles. CPU only: no GPU call."""
import itertools

import numpy as np

import merge_cases as MC
from conftest import pkg

D = pkg("decompose")
M = pkg("mesh")
G = pkg("meshgen")


def _pair_sets():
    sets = [MC.slabs([0.5]), MC.slabs([0.25, 0.5, 0.75]), MC.l_boxes(), MC.grid_boxes(),
            MC.cut_parts(G.noisy_icosphere(2, seed=3), [[1, 0, 0, -0.5], [0, 1, 0, -0.45], [0.3, 0.2, 0.93, -0.6]]),
            MC.cut_parts(G.staircase(8), [[0, 1, 0, -1.0], [0, 0, 1, -0.5], [1, 0, 0, -0.5]])]
    for parts in sets:
        for a, b in itertools.permutations(parts, 2):
            yield a, b


def test_seam_plane_matches_oracle(oracle):
    n = found = 0
    for a, b in _pair_sets():
        for tol in (1e-3, 1e-6):
            got = D.seam_plane(a, b, tol)
            ref = oracle.seam_plane(a, b, tol)
            assert (got is None) == (ref is None)
            if got is not None:
                assert np.array_equal(np.asarray(got), np.asarray(ref))
                found += 1
            n += 1
    assert n > 100 and found > 20


def test_seam_plane_reference_case():
    # merge.test.ts:36-37: the seam of the cube halves is the plane x = 0.5
    a, b = MC.slabs([0.5])
    s = D.seam_plane(a, b, 1e-3)
    assert s is not None and abs(abs(s[0]) - 1) < 1e-6 and abs(abs(s[3]) - 0.5) < 1e-6


def test_filtered_concat_matches_oracle(oracle):
    n = 0
    for a, b in _pair_sets():
        s = D.seam_plane(a, b, 1e-3)
        planes = ([s] if s else []) + [[0, 0, 1, -0.5], [1, 0, 0, -1.0]]
        for k in range(len(planes) + 1):
            got = D.filtered_concat(a.mesh, b.mesh, planes[:k], 1e-3)
            ref = oracle.filtered_concat(a.mesh, b.mesh, planes[:k], 1e-3)
            assert np.array_equal(got.tris, ref)
            assert np.array_equal(got.verts, np.concatenate([a.mesh.verts, b.mesh.verts]))
            n += 1
    assert n > 100


def test_filtered_concat_drops_the_seam():
    # both caps of the cube halves lie on x = 0.5 (8 boundary vertices each:
    # 6 triangles each) and go; nothing else does
    a, b = MC.slabs([0.5])
    m = D.filtered_concat(a.mesh, b.mesh, [[1, 0, 0, -0.5]], 1e-3)
    on = lambda x: int(np.all(np.abs(x.verts[x.tris][:, :, 0] - 0.5) < 1e-6, axis=1).sum())  # noqa: E731
    assert on(a.mesh) == 6 and on(b.mesh) == 6
    assert m.nt == a.mesh.nt + b.mesh.nt - 12


def test_seam_plane_and_filtered_concat_random_cuts(oracle):
    """Pieces of noisy icospheres and blobs cut by seeded random planes: every
    ordered pair's seam plane and filtered union equal the oracle's."""
    rng = np.random.default_rng(11)
    n = seams = 0
    meshes = [G.noisy_icosphere(2, seed=5), G.noisy_icosphere(3, seed=6), M.normalize(G.blob_mesh(5, 22, seed=7))[0]]
    for mesh in meshes:
        lo, hi = mesh.verts.min(0).astype(np.float64), mesh.verts.max(0).astype(np.float64)
        planes = []
        for _ in range(3):
            nrm = rng.normal(size=3)
            nrm /= np.linalg.norm(nrm)
            p = lo + rng.uniform(0.3, 0.7, 3) * (hi - lo)
            planes.append([nrm[0], nrm[1], nrm[2], -float(nrm @ p)])
        parts = MC.cut_parts(mesh, planes)
        for a, b in itertools.permutations(parts, 2):
            got = D.seam_plane(a, b, 1e-3)
            ref = oracle.seam_plane(a, b, 1e-3)
            assert (got is None) == (ref is None)
            if got is not None:
                assert np.array_equal(np.asarray(got), np.asarray(ref))
                seams += 1
            pl = ([got] if got else []) + [planes[0]]
            assert np.array_equal(D.filtered_concat(a.mesh, b.mesh, pl, 1e-3).tris,
                                  oracle.filtered_concat(a.mesh, b.mesh, pl, 1e-3))
            n += 1
    assert n > 60 and seams > 10, (n, seams)
