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
