"""Concave-edge planes on the GPU (cuacd_tree_concave_planes,
csrc/concave_kernels.cu) against the host restatement (cuacd_concave_planes)
and the oracle's restatement of src/cpu/concave.ts:25-92: the same planes bit
for bit, in the same order, for every mesh, reservoir size and seed —
including meshes with more concave edges than reservoir slots, where the
seeded LCG decides which edges are kept."""
import numpy as np
import pytest

from conftest import pkg
from fixtures import M, l_prism, square_torus, stairs

pytestmark = pytest.mark.gpu

D = pkg("decompose")
G = pkg("meshgen")
T = pkg("tree")


def _meshes():
    return [l_prism(), stairs(), G.staircase(8), G.staircase(12), G.staircase(8, wall_centroids=True), square_torus(),
            M.unit_cube(), M.l_shape(), G.noisy_icosphere(3, seed=1),
            M.normalize(G.blob_mesh(6, 26, seed=3))[0], M.normalize(G.blob_mesh(12, 40, seed=5))[0],
            G.carved_sphere(3, 3, seed=2)]


@pytest.mark.parametrize("n_edges", [1, 4, 16, 64])
def test_gpu_concave_planes_match_host_and_oracle(oracle, n_edges):
    g = T.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0)
    meshes = _meshes()
    for seeds in ([12345] * len(meshes), [7919 * 3 + k for k in range(len(meshes))], [3] * len(meshes)):
        got = g.concave_planes(meshes, n_edges, 0.005, 3.49, seeds)
        for m, s, p in zip(meshes, seeds, got):
            host = D.concave_planes(m, n_edges, 0.005, 3.49, s)
            ref = np.asarray(oracle.concave_planes(m, n_edges, 0.005, 3.49, s), np.float32).reshape(-1, 4)
            assert p.shape == host.shape == ref.shape
            assert np.array_equal(p.view(np.uint32), host.view(np.uint32))
            assert np.array_equal(p, ref)
    # more concave edges than slots somewhere, so the reservoir's LCG ran
    assert any(len(p) == 4 * n_edges or len(p) >= 2 * n_edges for p in got)


def test_gpu_concave_planes_reference_case():
    # tests/cpu.test.ts:89-95: the L prism's one concave edge gives 4 planes;
    # a convex mesh and the (convex-edged) L-shape box union give none
    g = T.GpuTree(width=3, width2=3, depth=1, nConcaveEdges=0)
    a, b, c = g.concave_planes([l_prism(), M.unit_cube(), M.l_shape()], 8)
    assert a.shape == (4, 4) and len(b) == 0 and len(c) == 0
