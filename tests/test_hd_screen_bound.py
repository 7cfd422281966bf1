"""The Hausdorff screen's error bound (csrc/hausdorff_kernels.cu, k_hd_screen)
against an emulation of its arithmetic on the CPU: |p - c|^2 screened as
|p|^2 + (|c|^2 - 2 p.c), the bracket a K = 16 contraction of bf16 hi/lo
splits ([p_hi, p_hi, p_lo, p_lo, 1, 1] x [-2c_hi, -2c_lo, -2c_hi, -2c_lo,
|c|^2_hi, |c|^2_lo]) accumulated in fp32. The tensor core's accumulation
order and rounding are not specified, so every emulated order and rounding
(sequential, pairwise, reversed, round-to-nearest and truncation, and the
exact sum rounded once) must stay within the kernel's bound
e = 2^-13 (|p|^2 + |c|^2 + 2 |p|_1 |c|_1) of the exact |p - c|^2, with |p|^2
and |c|^2 as fp32 dot products with or without fused multiply-adds. Points
near the origin, far from it (where |p|^2 and -2 p.c cancel) and at any
distance from the centroid. CPU only."""
from fractions import Fraction

import numpy as np
import pytest

f32 = np.float32


def bf16(x):
    """round to nearest even bfloat16 (8-bit significand), as __float2bfloat16_rn"""
    b = np.array([x], np.float32).view(np.uint32)[0]
    b = (int(b) + 0x7FFF + ((int(b) >> 16) & 1)) & 0xFFFF0000
    return np.array([b], np.uint32).view(np.float32)[0]


def split(x):
    h = bf16(x)
    return h, bf16(f32(x - h))


def rz(x):
    """float64 -> float32 rounded toward zero"""
    r = f32(x)
    if abs(float(r)) > abs(x):
        r = np.nextafter(r, f32(0.0))
    return f32(r)


def fma32(a, b, c):
    exact = Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))
    r = f32(float(exact))
    cand = [r, np.nextafter(r, f32(np.inf)), np.nextafter(r, f32(-np.inf))]
    return f32(min(cand, key=lambda x: (abs(Fraction(float(x)) - exact),
                                        int(np.array([x], np.float32).view(np.uint32)[0]) & 1)))


def dot_plain(a, b):
    return f32(f32(f32(a[0] * b[0]) + f32(a[1] * b[1])) + f32(a[2] * b[2]))


def dot_fma(a, b):
    r = f32(a[0] * b[0])
    r = fma32(a[1], b[1], r)
    return fma32(a[2], b[2], r)


def accumulations(terms):
    """the contraction's fp32 sum under several orders and roundings"""
    t = [f32(x) for x in terms]
    out = []
    for order in (t, t[::-1]):
        s = f32(0.0)
        for x in order:
            s = f32(s + x)
        out.append(s)
        s = f32(0.0)
        for x in order:
            s = rz(float(s) + float(x))
        out.append(s)
    level = t
    while len(level) > 1:
        level = [f32(level[i] + level[i + 1]) if i + 1 < len(level) else level[i] for i in range(0, len(level), 2)]
    out.append(level[0])
    out.append(f32(float(sum(Fraction(float(x)) for x in t))))
    return out


def screened(p, g, dot):
    cc = dot(g, g)
    ph = [split(p[i]) for i in range(3)]
    ch = [split(f32(f32(-2.0) * g[i])) for i in range(3)]
    cch = split(cc)
    a = [ph[0][0], ph[1][0], ph[2][0], ph[0][0], ph[1][0], ph[2][0], ph[0][1], ph[1][1], ph[2][1],
         ph[0][1], ph[1][1], ph[2][1], f32(1.0), f32(1.0), f32(0.0), f32(0.0)]
    b = [ch[0][0], ch[1][0], ch[2][0], ch[0][1], ch[1][1], ch[2][1], ch[0][0], ch[1][0], ch[2][0],
         ch[0][1], ch[1][1], ch[2][1], cch[0], cch[1], f32(0.0), f32(0.0)]
    terms = [f32(x * y) for x, y in zip(a, b)]  # bf16 x bf16 products are exact in fp32
    p2 = dot(p, p)
    p1 = f32(f32(abs(p[0]) + abs(p[1])) + abs(p[2]))
    c1 = f32(f32(abs(g[0]) + abs(g[1])) + abs(g[2]))
    e = f32(f32(1.220703125e-4) * f32(f32(p2 + cc) + f32(f32(f32(2.0) * p1) * c1)))
    return [f32(p2 + v) for v in accumulations(terms)], e


@pytest.mark.parametrize("seed", [0, 1])
def test_screen_error_within_bound(seed):
    rng = np.random.default_rng(seed)
    worst = 0.0
    for i in range(600):
        off = np.array([0.0, 0.0, 0.0]) if i % 3 == 0 else rng.choice([1.0, 1000.0, -500.0, 1.0e4]) * rng.normal(size=3)
        scale = 10.0 ** rng.uniform(-4, 1)
        g = (off + rng.normal(size=3) * scale).astype(np.float32)
        kind = i % 4
        if kind == 0:
            p = (g + rng.normal(size=3) * scale).astype(np.float32)
        elif kind == 1:  # the sample at the centroid or very close
            p = (g.astype(np.float64) + rng.normal(size=3) * scale * 1e-6).astype(np.float32)
        elif kind == 2:  # far apart
            p = (g + rng.normal(size=3) * scale * 1e3).astype(np.float32)
        else:
            p = g.copy()
        exact = sum((Fraction(float(p[k])) - Fraction(float(g[k]))) ** 2 for k in range(3))
        for dot in (dot_plain, dot_fma):
            qs, e = screened(p, g, dot)
            for q in qs:
                err = abs(Fraction(float(q)) - exact)
                assert err <= Fraction(float(e)), (p, g, float(q), float(exact), float(e))
                if e > 0:
                    worst = max(worst, float(err / Fraction(float(e))))
    # the bound is not loose by orders of magnitude on every input
    assert worst > 1e-3, worst
