"""The GPU ear test's orientation filters (csrc/cut_kernels.cu: orient_sign
and orient_ff), restated in IEEE float32 arithmetic on the CPU, against the
host clipper's double orient2 (csrc/plane_cut.cpp): wherever a filter
decides, its sign is the double result's sign. The filters carry the GPU
cut's bit-for-bit agreement with the host cut, so their error bounds are
checked here on adversarial inputs: near-collinear triples at many scales
and offsets, exactly collinear ones (double rounding noise), coordinates far
from the origin and tiny differences. CPU only.

float32 add, subtract and multiply are numpy's (round to nearest even, as
__fadd_rn / __fsub_rn / __fmul_rn); the fused multiply-add of the float-float
filter is exact arithmetic on fractions rounded once to float32."""
from fractions import Fraction

import numpy as np
import pytest

f32 = np.float32


def fma32(a, b, c):
    """__fmaf_rn: a * b + c rounded once to float32."""
    exact = Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))
    r = f32(float(exact))  # nearest double, then nearest float
    # correct a double rounding: pick the float nearest the exact value
    cand = [r, np.nextafter(r, f32(np.inf)), np.nextafter(r, f32(-np.inf))]
    best = min(cand, key=lambda x: (abs(Fraction(float(x)) - exact), int(np.frombuffer(x.tobytes(), np.uint32)[0]) & 1))
    return f32(best)


def split(x):
    """Ring coordinates: hi = fl32(x), lo = fl32(x - hi) (x - hi exact in double)."""
    h = f32(x)
    return h, f32(x - float(h))


def orient2_double(a, b, c):
    return (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0])


def ring_diff(hb, lb, ha, la):
    return f32(f32(hb - ha) + f32(lb - la))


def two_sum(a, b):
    s = f32(a + b)
    bv = f32(s - a)
    av = f32(s - bv)
    e = f32(f32(a - av) + f32(b - bv))
    return s, e


def ring_diff2(hb, lb, ha, la):
    s, e = two_sum(hb, f32(-ha))
    return s, f32(e + f32(lb - la))


def float_filter(A, B, Cc):
    """orient_sign's first stage: +1 / -1, or None when undecided."""
    d1 = ring_diff(B[0][0], B[0][1], A[0][0], A[0][1])
    d2 = ring_diff(Cc[1][0], Cc[1][1], A[1][0], A[1][1])
    d3 = ring_diff(B[1][0], B[1][1], A[1][0], A[1][1])
    d4 = ring_diff(Cc[0][0], Cc[0][1], A[0][0], A[0][1])
    p1, p2 = f32(d1 * d2), f32(d3 * d4)
    o = f32(p1 - p2)
    S = max(abs(A[0][0]), abs(A[1][0]), abs(B[0][0]), abs(B[1][0]), abs(Cc[0][0]), abs(Cc[1][0]))
    if not S < f32(1e15):
        return None, S
    u = f32(5.9604645e-8)
    eb = f32(f32(f32(8.0) * u * f32(abs(p1) + abs(p2))) +
             f32(f32(f32(f32(8.0) * u * u) * S) * f32(f32(abs(d1) + abs(d2)) + f32(abs(d3) + abs(d4)))))
    if eb > f32(1e-30):
        if o > eb:
            return 1, S
        if o < -eb:
            return -1, S
    return None, S


def ff_filter(A, B, Cc, S):
    """orient_ff: +1 / -1, or None when undecided."""
    s1, r1 = ring_diff2(B[0][0], B[0][1], A[0][0], A[0][1])
    s2, r2 = ring_diff2(Cc[1][0], Cc[1][1], A[1][0], A[1][1])
    s3, r3 = ring_diff2(B[1][0], B[1][1], A[1][0], A[1][1])
    s4, r4 = ring_diff2(Cc[0][0], Cc[0][1], A[0][0], A[0][1])
    p1 = f32(s1 * s2)
    q1 = fma32(s1, s2, -p1)
    p2 = f32(s3 * s4)
    q2 = fma32(s3, s4, -p2)
    c1 = f32(f32(f32(s1 * r2) + f32(r1 * s2)) + f32(r1 * r2))
    c2 = f32(f32(f32(s3 * r4) + f32(r3 * s4)) + f32(r3 * r4))
    h, g = two_sum(p1, f32(-p2))
    tail = f32(f32(f32(q1 - q2) + f32(c1 - c2)) + g)
    o = f32(h + tail)
    u2 = f32(3.5527137e-15)
    ss = f32(f32(abs(s1) + abs(s2)) + f32(abs(s3) + abs(s4)))
    E = f32(f32(f32(20.0) * u2) * f32(abs(p1) + abs(p2)))
    E = f32(E + f32(f32(f32(24.0) * u2 * S) * ss))
    E = f32(E + f32(f32(f32(f32(128.0) * u2) * f32(5.9604645e-8) * S) * S))
    E = f32(E + f32(f32(7.2e-43) * f32(ss + f32(1.0))))
    E = f32(E * f32(1.02))
    if o > E:
        return 1
    if o < -E:
        return -1
    return None


def cases(rng, n):
    """Triples (a, b, c) in double: random, near-collinear at several
    scales, exactly collinear in exact arithmetic, and offset far out."""
    out = []
    for _ in range(n):
        kind = rng.integers(0, 5)
        off = rng.choice([0.0, 1.0, 37.5, -1000.0, 3.0e5]) * rng.uniform(0.5, 1.5, 2)
        scale = 10.0 ** rng.uniform(-6, 1)
        a = off + rng.normal(size=2) * scale
        d = rng.normal(size=2) * scale
        if kind == 0:
            b, c = a + d, a + rng.normal(size=2) * scale
        elif kind == 1:  # near-collinear: c on the line through a, b plus a tiny normal offset
            t = rng.uniform(-2, 3)
            nrm = np.array([-d[1], d[0]])
            c = a + t * d + nrm * 10.0 ** rng.uniform(-18, -6)
            b = a + d
        elif kind == 2:  # collinear in exact arithmetic, rounded to double
            b = a + d
            c = a + rng.uniform(-2, 3) * d
        elif kind == 3:  # three points on an axis-parallel line (slab sides)
            y = a[1]
            b = np.array([a[0] + d[0], y])
            c = np.array([a[0] + rng.uniform(-2, 3) * d[0], y + 10.0 ** rng.uniform(-20, -8) * rng.choice([-1, 1])])
        else:  # tiny triangle far from the origin
            b = a + d * 1e-7
            c = a + rng.normal(size=2) * scale * 1e-7
        out.append((a, b, c))
    return out


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_filters_agree_with_double_where_they_decide(seed):
    rng = np.random.default_rng(seed)
    decided1 = decided2 = undecided = 0
    for a, b, c in cases(rng, 3000):
        a = (float(a[0]), float(a[1]))
        b = (float(b[0]), float(b[1]))
        c = (float(c[0]), float(c[1]))
        r = orient2_double(a, b, c)
        want = 1 if r > 0 else (-1 if r < 0 else 0)
        A = (split(a[0]), split(a[1]))
        B = (split(b[0]), split(b[1]))
        Cc = (split(c[0]), split(c[1]))
        s1, S = float_filter(A, B, Cc)
        if s1 is not None:
            decided1 += 1
            assert s1 == want, (a, b, c, r, s1)
            continue
        if not S < f32(1e15):
            undecided += 1
            continue
        s2 = ff_filter(A, B, Cc, S)
        if s2 is not None:
            decided2 += 1
            assert s2 == want, (a, b, c, r, s2)
        else:
            undecided += 1
    # the cases reach all three stages
    assert decided1 > 500 and decided2 > 100 and undecided > 100, (decided1, decided2, undecided)
