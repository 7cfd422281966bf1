"""Seeded synthetic meshes for the benchmark workloads.

* ``icosphere`` / ``noisy_icosphere``: subdivided icosahedron, optionally
  displaced radially by seeded uniform noise and normalised to the unit cube.
* ``staircase``: the union of n axis-aligned boxes (width 1, depth 0.25,
  heights k * 0.125), welded into one closed manifold.
* ``random_planes``: seeded candidate planes through a mesh.
* ``blob_mesh``: an isosurface of a sum of Gaussian blobs, meshed by marching
  tetrahedra (see ``isosurface``).
"""
from __future__ import annotations

import numpy as np

from .mesh import Mesh


def icosphere(level: int) -> Mesh:
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(level):
        cache = {}

        def mid(a, b):
            k = (min(a, b), max(a, b))
            if k not in cache:
                p = verts[a] + verts[b]
                verts.append(p / np.linalg.norm(p))
                cache[k] = len(verts) - 1
            return cache[k]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return Mesh(np.array(verts, np.float32), np.array(faces, np.uint32))


def noisy_icosphere(level: int = 4, noise: float = 0.15, seed: int = 0) -> Mesh:
    """Icosphere with every vertex displaced radially by U[-noise, noise] of
    the radius, then uniformly scaled into the unit cube [0, 1]^3."""
    m = icosphere(level)
    rng = np.random.default_rng(seed)
    v = m.verts.astype(np.float64)
    v = v * (1.0 + rng.uniform(-noise, noise, size=(len(v), 1)))
    lo, hi = v.min(0), v.max(0)
    v = (v - lo) / (hi - lo).max()
    return Mesh(v.astype(np.float32), m.tris)


def random_planes(m: Mesh, n: int, seed: int = 0) -> np.ndarray:
    """n planes (a, b, c, d) with unit normals uniform on the sphere and
    offsets uniform over the mesh's extent along each normal."""
    rng = np.random.default_rng(seed)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    proj = m.verts.astype(np.float64) @ nrm.T  # (nv, n)
    lo, hi = proj.min(0), proj.max(0)
    off = lo + rng.uniform(0.0, 1.0, size=n) * (hi - lo)
    return np.concatenate([nrm, -off[:, None]], axis=1).astype(np.float32)


def staircase(n_steps: int = 8, width: float = 1.0, depth: float = 0.25, rise: float = 0.125,
              wall_centroids: bool = False) -> Mesh:
    """Union of n_steps boxes [0, width] x [(k-1) depth, k depth] x [0, k rise],
    k = 1..n_steps, as one closed manifold without T-junctions.

    Each side wall (x = 0 and x = width) is split into one polygon per box
    column: a quad for the first column and a pentagon (the previous
    column's top corner on its left edge) for the others, fanned from the
    bottom-left corner. Treads, risers, the back wall and the bottom are one
    quad per box. For n_steps = 8 this is 96 triangles over 50 vertices.

    wall_centroids: every side-wall triangle is split at its centroid into
    three, so the two large walls carry interior vertices. For n_steps = 8
    that adds 46 vertices: 188 triangles over 96 vertices (a closed genus-0
    triangulation has 2 V - 4 triangles), the staircase configuration's
    triangle count. The solid, and so every hull, is the same.
    """
    ys = [k * depth for k in range(n_steps + 1)]
    hs = [k * rise for k in range(n_steps + 1)]
    verts = []
    index = {}

    def vid(x, y, z):
        key = (round(x, 9), round(y, 9), round(z, 9))
        if key not in index:
            index[key] = len(verts)
            verts.append((x, y, z))
        return index[key]

    tris = []

    def quad(a, b, c, d):  # counter-clockwise seen from outside
        tris.extend([(a, b, c), (a, c, d)])

    for side, x in ((0, 0.0), (1, width)):
        for k in range(1, n_steps + 1):
            y0, y1, h = ys[k - 1], ys[k], hs[k]
            poly = [(y0, 0.0), (y1, 0.0), (y1, h), (y0, h)]
            if k > 1:
                poly.append((y0, hs[k - 1]))
            ids = [vid(x, y, z) for y, z in poly]
            # outward normal of the x = 0 wall is -x: the (y, z) polygon above
            # is counter-clockwise seen from +x, so wall 0 is reversed
            for i in range(1, len(ids) - 1):
                t = (ids[0], ids[i], ids[i + 1])
                t = t if side == 1 else (t[0], t[2], t[1])
                if wall_centroids:
                    p = [verts[j] for j in t]
                    c = len(verts)
                    verts.append(tuple(sum(q[a] for q in p) / 3.0 for a in range(3)))
                    tris.extend([(t[0], t[1], c), (t[1], t[2], c), (t[2], t[0], c)])
                else:
                    tris.append(t)
    for k in range(1, n_steps + 1):
        y0, y1, h = ys[k - 1], ys[k], hs[k]
        # tread (+z)
        quad(vid(0, y0, h), vid(width, y0, h), vid(width, y1, h), vid(0, y1, h))
        # riser facing -y, from the previous tread (or the floor) up to h
        hp = hs[k - 1]
        quad(vid(0, y0, hp), vid(width, y0, hp), vid(width, y0, h), vid(0, y0, h))
        # bottom (-z)
        quad(vid(0, y0, 0), vid(0, y1, 0), vid(width, y1, 0), vid(width, y0, 0))
    # back wall (+y) at y = n_steps * depth
    yb, hb = ys[-1], hs[-1]
    quad(vid(0, yb, 0), vid(0, yb, hb), vid(width, yb, hb), vid(width, yb, 0))
    return _orient_outward(Mesh(np.array(verts, np.float32), np.array(tris, np.uint32)))


def _orient_outward(m: Mesh) -> Mesh:
    from .mesh import signed_volume

    if signed_volume(m) < 0:
        return Mesh(m.verts, m.tris[:, [0, 2, 1]])
    return m


# ---------------------------------------------------------------------------
# Gaussian-blob isosurfaces (marching tetrahedra)

# The six tetrahedra of the Kuhn split of a unit cube: corner offsets along
# each permutation (a, b, c) of the axes from (0,0,0) to (1,1,1). Neighbouring
# cubes split their shared faces the same way, so the surface is conforming.
_KUHN = []
for _a, _b, _c in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
    _p = [0, 0, 0]
    _tet = [tuple(_p)]
    for _ax in (_a, _b, _c):
        _p[_ax] = 1
        _tet.append(tuple(_p))
    _KUHN.append(_tet)


def isosurface(field: np.ndarray, lo, hi, level: float) -> Mesh:
    """Closed, outward-wound surface {field = level} of a sampled field
    (inside = field > level) by marching tetrahedra on the Kuhn split of
    each grid cube. Vertices sit on grid edges and are shared by edge, so the
    mesh is a closed 2-manifold when the field is below the level on the
    grid's boundary. Values equal to the level count as outside."""
    f = np.asarray(field, np.float64)
    nx, ny, nz = f.shape
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    step = (hi - lo) / (np.array([nx, ny, nz]) - 1)
    ins = f > level
    # cube origins
    ci, cj, ck = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1), np.arange(nz - 1), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    # keep cubes whose 8 corners are not all on one side
    corners = np.stack([ins[ci + dx, cj + dy, ck + dz] for dx in (0, 1) for dy in (0, 1) for dz in (0, 1)], 1)
    mixed = corners.any(1) & ~corners.all(1)
    ci, cj, ck = ci[mixed], cj[mixed], ck[mixed]

    def gid(i, j, k):
        return (i * ny + j) * nz + k

    tets = np.concatenate([np.stack([gid(ci + o[0], cj + o[1], ck + o[2]) for o in tet], 1) for tet in _KUHN])
    s = ins.ravel()[tets]
    nin = s.sum(1)
    fr = f.ravel()
    tris_e = []  # triangles as (edge a, edge b) pairs of grid ids, shape (n, 3, 2)
    orient = []  # (inside id, outside id) of each triangle, to wind it outward
    # one corner alone on its side: one triangle on its three edges
    for lone_inside in (True, False):
        sel = nin == (1 if lone_inside else 3)
        t = tets[sel]
        st = s[sel] if lone_inside else ~s[sel]
        k = np.argmax(st, 1)
        lone = t[np.arange(len(t)), k]
        others = np.stack([t[np.arange(len(t)), (k + d) % 4] for d in (1, 2, 3)], 1)
        tris_e.append(np.stack([np.stack([lone, others[:, q]], 1) for q in range(3)], 1))
        ins_id, out_id = (lone, others[:, 0]) if lone_inside else (others[:, 0], lone)
        orient.append(np.stack([ins_id, out_id], 1))
    # two inside, two outside: a quad on the four crossing edges
    sel = nin == 2
    t = tets[sel]
    st = s[sel]
    order = np.argsort(~st, axis=1, kind="stable")  # inside corners first
    i1, i2 = t[np.arange(len(t)), order[:, 0]], t[np.arange(len(t)), order[:, 1]]
    o1, o2 = t[np.arange(len(t)), order[:, 2]], t[np.arange(len(t)), order[:, 3]]
    q = [np.stack([i1, o1], 1), np.stack([i1, o2], 1), np.stack([i2, o2], 1), np.stack([i2, o1], 1)]
    tris_e.append(np.stack([q[0], q[1], q[2]], 1))
    tris_e.append(np.stack([q[0], q[2], q[3]], 1))
    orient.append(np.stack([i1, o1], 1))
    orient.append(np.stack([i1, o1], 1))
    E = np.concatenate(tris_e)  # (n, 3, 2)
    O = np.concatenate(orient)
    # weld by grid edge
    a, b = np.minimum(E[..., 0], E[..., 1]), np.maximum(E[..., 0], E[..., 1])
    key = a.astype(np.int64) * (nx * ny * nz) + b
    uk, inv = np.unique(key.ravel(), return_inverse=True)
    ea, eb = uk // (nx * ny * nz), uk % (nx * ny * nz)

    def pos(g):
        i, r = np.divmod(g, ny * nz)
        j, k = np.divmod(r, nz)
        return lo + np.stack([i, j, k], 1) * step

    fa, fb = fr[ea], fr[eb]
    tt = (level - fa) / (fb - fa)
    verts = pos(ea) + tt[:, None] * (pos(eb) - pos(ea))
    tris = inv.reshape(-1, 3)
    # wind outward: the normal points from the inside corner to the outside one
    v0, v1, v2 = verts[tris[:, 0]], verts[tris[:, 1]], verts[tris[:, 2]]
    nrm = np.cross(v1 - v0, v2 - v0)
    d = pos(O[:, 1]) - pos(O[:, 0])
    flip = (nrm * d).sum(1) < 0
    tris[flip] = tris[flip][:, [0, 2, 1]]
    return Mesh(verts.astype(np.float32), tris.astype(np.uint32))


def blob_field(n_blobs: int, grid: int, seed: int = 0, sigma=(0.15, 0.45)):
    """Sum of n seeded isotropic Gaussian blobs (centres uniform in [-1, 1]^3,
    sigma uniform in `sigma`, unit amplitude) sampled on a grid^3 lattice
    spanning the centres' box plus 3.2 sigma_max on every side."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1, 1, (n_blobs, 3))
    sg = rng.uniform(sigma[0], sigma[1], n_blobs)
    pad = 3.2 * sigma[1]
    lo, hi = np.full(3, -1 - pad), np.full(3, 1 + pad)
    ax = np.linspace(lo[0], hi[0], grid)
    f = np.zeros((grid, grid, grid))
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij", sparse=True)
    for k in range(n_blobs):
        f += np.exp(-((X - c[k, 0]) ** 2 + (Y - c[k, 1]) ** 2 + (Z - c[k, 2]) ** 2) / (2 * sg[k] ** 2))
    return f, lo, hi


def blob_mesh(n_blobs: int = 24, grid: int = 160, seed: int = 0, level: float = 0.5, sigma=(0.15, 0.45)) -> Mesh:
    """Isosurface (level 0.5) of a sum of Gaussian blobs, marching tetrahedra."""
    f, lo, hi = blob_field(n_blobs, grid, seed, sigma)
    # a sample exactly at the level would put a vertex on a grid point
    f = np.where(f == level, np.nextafter(level, 0.0), f)
    return isosurface(f, lo, hi, level)


def blob_batch(n_meshes: int = 256, seed: int = 0, tri_range=(500, 60000)):
    """Uneven batch: blob counts uniform in 2..32, each mesh's grid chosen so
    the triangle counts are log-uniform in tri_range (the count of a
    marching-tetrahedra surface grows with the square of the grid size)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_meshes):
        nb = int(rng.integers(2, 33))
        target = float(np.exp(rng.uniform(np.log(tri_range[0]), np.log(tri_range[1]))))
        g0 = 24
        m0 = blob_mesh(nb, g0, seed=seed * 100003 + k)
        g = int(np.clip(round(g0 * np.sqrt(target / max(m0.nt, 1))), 8, 400))
        out.append(blob_mesh(nb, g, seed=seed * 100003 + k))
    return out


def carved_sphere(level: int = 4, n_holes: int = 3, seed: int = 0) -> Mesh:
    """A unit sphere minus n_holes seeded spheres (centres near the surface,
    radii 0.2..0.6), meshed from its signed distance by marching tetrahedra
    on a grid sized so the triangle count is near an icosphere of `level`
    (20 * 4^level)."""
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n_holes, 3))
    c = d / np.linalg.norm(d, axis=1, keepdims=True) * rng.uniform(0.6, 1.1, (n_holes, 1))
    r = rng.uniform(0.2, 0.6, n_holes)

    def field(g):
        ax = np.linspace(-1.25, 1.25, g)
        X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij", sparse=True)
        sd = np.sqrt(X * X + Y * Y + Z * Z) - 1.0
        for k in range(n_holes):
            hole = np.sqrt((X - c[k, 0]) ** 2 + (Y - c[k, 1]) ** 2 + (Z - c[k, 2]) ** 2) - r[k]
            sd = np.maximum(sd, -hole)
        f = -sd
        return np.where(f == 0.0, -1e-12, f)

    target = 20 * 4 ** level
    g0 = 24
    m0 = isosurface(field(g0), (-1.25,) * 3, (1.25,) * 3, 0.0)
    g = int(np.clip(round(g0 * np.sqrt(target / max(m0.nt, 1))), 8, 400))
    return isosurface(field(g), (-1.25,) * 3, (1.25,) * 3, 0.0)


def serving_mix(n: int, seed: int = 0):
    """The serving workload's request mix: 40% staircases of 4..16 steps,
    40% Gaussian-blob isosurfaces of 2k..60k triangles, 20% icospheres of
    level 3..5 carved by 1..6 spheres; thresholds drawn from {0.05, 0.1}.
    Returns (kind, mesh, threshold) triples."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        u = rng.uniform()
        thr = float(rng.choice([0.05, 0.1]))
        if u < 0.4:
            out.append(("staircase", staircase(int(rng.integers(4, 17))), thr))
        elif u < 0.8:
            nb = int(rng.integers(2, 33))
            target = float(np.exp(rng.uniform(np.log(2000), np.log(60000))))
            m0 = blob_mesh(nb, 24, seed=seed * 7919 + k)
            g = int(np.clip(round(24 * np.sqrt(target / max(m0.nt, 1))), 8, 400))
            out.append(("blob", blob_mesh(nb, g, seed=seed * 7919 + k), thr))
        else:
            out.append(("carved", carved_sphere(int(rng.integers(3, 6)), int(rng.integers(1, 7)), seed=seed * 7919 + k), thr))
    return out
