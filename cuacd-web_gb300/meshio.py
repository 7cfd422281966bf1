"""Mesh file formats at the edge of the decomposition (src/mesh.ts:166-242):
binary and ASCII STL (welded by exact position), simple OBJ, and the OBJ
writer of the parts.

    mesh = parse_stl(open("part.stl", "rb").read())
    text = to_obj([p.hull for p in decompose(mesh).parts])

Numbers are written as JavaScript prints them (Number.prototype.toString of
the float32 value widened to double), so the OBJ text is the reference's
byte for byte.
"""
from __future__ import annotations

import re
import struct
from decimal import Decimal

import numpy as np

from .mesh import Mesh

_VERTEX = re.compile(rb"vertex\s+([-+0-9.eE]+)\s+([-+0-9.eE]+)\s+([-+0-9.eE]+)")


def _looks_binary(buf: bytes) -> bool:
    if len(buf) < 84:
        return False
    n = struct.unpack_from("<I", buf, 80)[0]
    return 84 + n * 50 == len(buf)


def parse_stl(buf: bytes) -> Mesh:
    """parseSTL (src/mesh.ts:166-187): binary unless the header starts with
    "solid" and the size does not match the binary layout."""
    buf = bytes(buf)
    head = buf[:80].decode("utf-8", errors="replace")
    binary = not (head.lstrip().startswith("solid") and not _looks_binary(buf))
    if binary:
        n = struct.unpack_from("<I", buf, 80)[0]
        rec = np.dtype([("n", "<f4", 3), ("v", "<f4", 9), ("a", "<u2")])
        tri = np.frombuffer(buf, rec, count=n, offset=84)
        pos = tri["v"].astype(np.float64).reshape(-1)
    else:
        vals = []
        for m in _VERTEX.finditer(buf):
            vals.extend(_js_number(g.decode()) for g in m.groups())
        pos = np.array(vals, np.float64)
    return weld(pos)


_JS_DEC = re.compile(r"[+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|[+-]?Infinity")
_JS_INT = re.compile(r"\s*([+-]?\d+)")


def _js_number(s: str) -> float:
    """Unary + on a string (ECMAScript StringToNumber): surrounding white
    space ignored, "" is 0, anything that is not a decimal or 0x/0o/0b
    literal is NaN."""
    t = s.strip()
    if t == "":
        return 0.0
    for pre, base in (("0x", 16), ("0o", 8), ("0b", 2)):
        if t[:2].lower() == pre:
            try:
                return float(int(t[2:], base)) if t[2:].isalnum() else float("nan")
            except ValueError:
                return float("nan")
    if not _JS_DEC.fullmatch(t):
        return float("nan")
    return float(t.replace("Infinity", "inf"))


def _js_parse_int(s: str):
    """parseInt(s, 10): the leading integer, None (NaN) when there is none."""
    m = _JS_INT.match(s)
    return int(m.group(1)) if m else None


def weld(pos) -> Mesh:
    """weld (src/mesh.ts:196-212): one vertex per distinct (x, y, z) value,
    in first-appearance order; float32 after welding."""
    p = np.asarray(pos, np.float64).reshape(-1, 3)
    index = {}
    verts = []
    tris = np.empty(len(p), np.uint32)
    for i, (x, y, z) in enumerate(p):
        # -0 and 0 print alike in the reference's string key
        k = (x + 0.0, y + 0.0, z + 0.0)
        j = index.get(k)
        if j is None:
            j = len(verts)
            index[k] = j
            verts.append((x, y, z))
        tris[i] = j
    v = np.array(verts, np.float32).reshape(-1, 3)
    return Mesh(v, tris.reshape(-1, 3))


def parse_obj(text: str) -> Mesh:
    """parseOBJ (src/mesh.ts:215-229): "v" and "f" lines, polygons fanned
    from their first vertex, texture/normal indices ignored; indices stored
    as uint32 as a Uint32Array stores them (NaN as 0, negatives wrapped)."""
    verts, tris = [], []
    for line in text.split("\n"):
        if line.startswith("v "):
            p = re.split(r"\s+", line)
            p += [None] * (4 - len(p))
            verts.extend(_js_number(x) if x is not None else float("nan") for x in p[1:4])
        elif line.startswith("f "):
            idx = []
            for tok in re.split(r"\s+", line.strip())[1:]:
                k = _js_parse_int(tok.split("/")[0])
                idx.append(0 if k is None else (k - 1) % (1 << 32))
            for i in range(1, len(idx) - 1):
                tris.extend((idx[0], idx[i], idx[i + 1]))
    v = np.array(verts, np.float32).reshape(-1, 3)
    t = np.array(tris, np.uint64).astype(np.uint32).reshape(-1, 3)
    return Mesh(v, t)


def js_number_string(x: float) -> str:
    """Number.prototype.toString() of a double (ECMAScript Number::toString):
    the shortest digits that round-trip (as repr finds them), written plainly
    for decimal exponents from -7 to 20 and as d.ddde+n otherwise."""
    x = float(x)
    if x != x:
        return "NaN"
    if x == 0:
        return "0"
    if x < 0:
        return "-" + js_number_string(-x)
    if x == float("inf"):
        return "Infinity"
    d = Decimal(repr(x)).normalize()
    _, digs, exp = d.as_tuple()
    digits = "".join(map(str, digs))
    k = len(digits)
    n = k + exp  # the value is 0.digits x 10^n
    if k <= n <= 21:
        return digits + "0" * (n - k)
    if 0 < n <= 21:
        return digits[:n] + "." + digits[n:]
    if -6 < n <= 0:
        return "0." + "0" * (-n) + digits
    e = n - 1
    sign = "+" if e >= 0 else "-"
    return (digits if k == 1 else digits[0] + "." + digits[1:]) + "e" + sign + str(abs(e))


def to_obj(parts) -> str:
    """toOBJ (src/mesh.ts:231-242): one "o part_i" group per mesh, indices
    offset across groups."""
    out = []
    base = 1
    for i, m in enumerate(parts):
        out.append(f"o part_{i}")
        v = np.asarray(m.verts, np.float32).reshape(-1, 3)
        for x, y, z in v:
            out.append(f"v {js_number_string(float(x))} {js_number_string(float(y))} {js_number_string(float(z))}")
        for a, b, c in np.asarray(m.tris, np.uint32).reshape(-1, 3):
            out.append(f"f {int(a) + base} {int(b) + base} {int(c) + base}")
        base += v.shape[0]
    return "\n".join(out) + "\n"
