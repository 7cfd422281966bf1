"""Mesh file formats (cuacd-web_gb300/meshio.py against src/mesh.ts:166-242):
STL (binary and ASCII, welded by exact position), OBJ in and out, and
JavaScript's number printing in the OBJ writer. CPU only."""
import os
import struct

import numpy as np
import pytest

from conftest import pkg
from fixtures import M, stairs

IO = pkg("meshio")
G = pkg("meshgen")
Mesh = pkg("mesh").Mesh


def _stl_binary(m, header=b"binary"):
    v = m.verts.astype(np.float32)
    out = [header.ljust(80, b"\0"), struct.pack("<I", len(m.tris))]
    for a, b, c in m.tris:
        out.append(struct.pack("<3f", 0, 0, 0) + v[[a, b, c]].tobytes() + b"\0\0")
    return b"".join(out)


def _stl_ascii(m):
    lines = ["solid test"]
    for a, b, c in m.tris:
        lines.append("facet normal 0 0 0\n outer loop")
        for i in (a, b, c):
            x, y, z = (repr(float(t)) for t in m.verts[i])
            lines.append(f"  vertex {x} {y} {z}")
        lines.append(" endloop\nendfacet")
    lines.append("endsolid test")
    return "\n".join(lines).encode()


@pytest.mark.parametrize("m", [M.unit_cube(), stairs(), G.staircase(8), G.noisy_icosphere(2, seed=3)])
def test_stl_binary_and_ascii_weld_back(m):
    for buf in (_stl_binary(m), _stl_binary(m, b"solid but binary"), _stl_ascii(m)):
        r = IO.parse_stl(buf)
        # vertices in first-appearance order over the triangle soup
        order = []
        for i in m.tris.reshape(-1):
            if i not in order:
                order.append(int(i))
        assert np.array_equal(r.verts, m.verts[order])
        remap = {o: k for k, o in enumerate(order)}
        assert np.array_equal(r.tris, np.vectorize(remap.get)(m.tris).astype(np.uint32))
        assert M.is_closed(r)


def test_stl_welds_by_exact_position():
    # -0 and 0 are one vertex (the reference keys by the printed number)
    soup = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0, -0.0, 0, 0, 0, 1, 0, 0, 0, 1], np.float64)
    r = IO.weld(soup)
    assert r.verts.shape == (4, 3)
    assert r.tris.tolist() == [[0, 1, 2], [0, 2, 3]]


def test_obj_round_trip_and_fans():
    parts = [M.unit_cube(), stairs()]
    text = IO.to_obj(parts)
    assert text.startswith("o part_0\nv 0 0 0\n")
    back = IO.parse_obj(text)
    assert back.verts.shape[0] == sum(p.verts.shape[0] for p in parts)
    assert np.array_equal(back.verts[:8], parts[0].verts)
    assert np.array_equal(back.tris[12:], parts[1].tris + 8)
    # a quad with texture/normal indices fans into two triangles
    q = IO.parse_obj("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1/1/1 2/2/2 3/3/3 4/4/4\n")
    assert q.tris.tolist() == [[0, 1, 2], [0, 2, 3]]


@pytest.mark.parametrize("x,s", [(1.0, "1"), (100.0, "100"), (0.5, "0.5"), (-3.25, "-3.25"), (0.0, "0"),
                                 (float(np.float32(0.1)), "0.10000000149011612"), (1e21, "1e+21"),
                                 (1e20, "100000000000000000000"), (1e-6, "0.000001"), (1e-7, "1e-7"),
                                 (1.5e-7, "1.5e-7"), (1e-5, "0.00001"), (2.0 ** 53, "9007199254740992"),
                                 (5e-324, "5e-324"), (1.7976931348623157e308, "1.7976931348623157e+308")])
def test_js_number_printing(x, s):
    assert IO.js_number_string(x) == s


def test_reference_stl_fixture_loads():
    # the reference's own test mesh (its tests/data/49160.stl, committed as a
    # fixture): closed after welding (decompose.test.ts:52-55)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "49160.stl")
    with open(path, "rb") as f:
        m = IO.parse_stl(f.read())
    assert m.tris.shape[0] > 0
    assert M.is_closed(m)
