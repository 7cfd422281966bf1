"""Part sets for the merge pass tests (tests/merge.test.ts:16-31 and more)."""
import numpy as np

from conftest import pkg

D = pkg("decompose")
M = pkg("mesh")
G = pkg("meshgen")


def part(m):
    """A part with its CPU hull (merge.test.ts:16-19: convexHull of the mesh's
    vertices, wound outward by the sign of its volume as compactHull does,
    hull.ts:157-185), mesh and hull volume, Hausdorff 0."""
    hv, ht = D.quickhull(m.verts.astype(np.float64))
    hull = M.Mesh(hv.astype(np.float32), ht.astype(np.uint32))
    if M.signed_volume(hull) < 0:
        hull = M.Mesh(hull.verts, np.ascontiguousarray(hull.tris[:, [0, 2, 1]]))
    return D.Part(mesh=m, hull=hull, meshVol=M.volume(m), hullVol=M.volume(hull), hausdorff=0.0)


def slabs(cuts):
    """The unit cube cut at x = c for each c, the negative halves in order and
    the rest last (merge.test.ts:20-31)."""
    rest = M.unit_cube()
    out = []
    for x in cuts:
        pos, neg = D.plane_cut(rest, [1, 0, 0, -x])
        out.append(part(neg))
        rest = pos
    out.append(part(rest))
    return out


def l_boxes():
    """The two boxes of an L-shape (merge.test.ts:56-63)."""
    return [part(M.make_box([0, 0, 0], [1, 1, 1])), part(M.make_box([1, 0, 0], [2, 1, 0.5]))]


def grid_boxes():
    """A 2 x 2 x 1 block of unit boxes and a detached box: merges across
    rounds, seams on different planes, one pair rejected by its bounding-box
    gap."""
    boxes = [M.make_box([i, j, 0], [i + 1, j + 1, 1]) for i in range(2) for j in range(2)]
    boxes.append(M.make_box([3.5, 0, 0], [4.5, 1, 1]))
    return [part(b) for b in boxes]


def cut_parts(mesh, planes):
    """The pieces of mesh cut successively by each plane (every piece cut by
    the next plane where it splits)."""
    pieces = [mesh]
    for pl in planes:
        nxt = []
        for p in pieces:
            try:
                a, b = D.plane_cut(p, pl)
                nxt += [a, b]
            except pkg("tree").CuacdError:
                nxt.append(p)
        pieces = nxt
    return [part(p) for p in pieces]
