"""The double-float pass's interval rule (k_prec_df), checked on the CPU.

For every axis the pass forms the six projections in double-float arithmetic
(pairs of floats) with a bound W on |double-float - exact| + |FP64 - exact|,
and decides the axis from the intervals [v - 2(W + 2^-23 |v|), v + 2(W +
2^-23 |v|)], v = hi + lo rounded: the FP64 pass's value of each projection
must lie inside. This replays the kernel's float arithmetic operation for
operation: round-to-nearest sums and products in numpy float32 (correctly
rounded), fused multiply-adds and the directed roundings of the bounds
(__fadd_ru, __fmul_ru, __fmaf_ru, __fsub_rd) as exact rationals rounded to
float32. The FP64 values follow the FP64 pass's formula (relative vertices,
edges, cross products, dot products in the reference's operation order,
src/utils/utils.cpp:97-169, one rounding per operation). Inputs: random
triangle pairs, nearly coplanar ones and exactly coplanar ones, at relative
extents across [2^-18, 2^18], and at the ends of the pass's range [2^-20,
2^20] with collinear triangles, shared vertices and shared edges; the check
covers every axis of each pair, not only the axes a pass would visit.
"""
from fractions import Fraction as Fr

import numpy as np

F = np.float32
_UP, _DN = F(np.inf), F(-np.inf)


def _exact(x) -> Fr:
    return Fr(float(x))


def _round(x: Fr, mode: str) -> np.float32:
    """float32 of the rational x rounded up ('ru'), down ('rd') or to nearest even ('rn')."""
    if x == 0:
        return F(0.0)
    f = F(float(x))
    while _exact(f) < x:
        f = np.nextafter(f, _UP)
    while _exact(np.nextafter(f, _DN)) >= x:
        f = np.nextafter(f, _DN)
    if mode == "ru":
        return f
    lo = f if _exact(f) == x else np.nextafter(f, _DN)
    if mode == "rd" or lo == f:
        return lo
    dlo, dhi = x - _exact(lo), _exact(f) - x
    if dlo != dhi:
        return lo if dlo < dhi else f
    return lo if (int(lo.view(np.uint32)) & 1) == 0 else f


def fma_rn(a, b, c):
    return _round(_exact(a) * _exact(b) + _exact(c), "rn")


def fma_ru(a, b, c):
    return _round(_exact(a) * _exact(b) + _exact(c), "ru")


def add_ru(a, b):
    return _round(_exact(a) + _exact(b), "ru")


def sub_rd(a, b):
    return _round(_exact(a) - _exact(b), "rd")


def mul_ru(a, b):
    return _round(_exact(a) * _exact(b), "ru")


U, ETA, GROW = F(2.0 ** -44), F(2.0 ** -140), F(1.0 + 2.0 ** -20)


def two_sum(a, b):
    s = F(a + b)
    ap = F(s - b)
    bp = F(s - ap)
    return (s, F(F(a - ap) + F(b - bp)))


def fast_two_sum(a, b):
    s = F(a + b)
    return (s, F(b - F(s - a)))


def df_add(x, y):
    s, t = two_sum(x[0], y[0]), two_sum(x[1], y[1])
    v = fast_two_sum(s[0], F(s[1] + t[0]))
    return fast_two_sum(v[0], F(t[1] + v[1]))


def df_mul(x, y):
    ch = F(x[0] * y[0])
    cl1 = fma_rn(x[0], y[0], -ch)
    tl1 = fma_rn(x[0], y[1], F(x[1] * y[1]))
    cl2 = fma_rn(x[1], y[0], tl1)
    return fast_two_sum(ch, F(cl1 + cl2))


def df_abs(x):
    return add_ru(abs(x[0]), abs(x[1]))


def w_sum(a, b, c):
    return add_ru(fma_ru(U, df_abs(c), mul_ru(GROW, add_ru(a[1], b[1]))), ETA)


def b_sub(a, b):
    c = df_add(a[0], (-b[0][0], -b[0][1]))
    return (c, w_sum(a, b, c))


def b_add(a, b):
    c = df_add(a[0], b[0])
    return (c, w_sum(a, b, c))


def b_mul(a, b):
    c = df_mul(a[0], b[0])
    w = fma_ru(df_abs(a[0]), b[1], mul_ru(df_abs(b[0]), a[1]))
    w = fma_ru(mul_ru(F(2.0), a[1]), b[1], w)
    return (c, add_ru(fma_ru(U, df_abs(c), mul_ru(GROW, w)), ETA))


def b_rel(a, b):
    d = two_sum(a, -b)
    return (d, mul_ru(F(2.0 ** -53), df_abs(d)))


def b3_sub(x, y):
    return [b_sub(x[i], y[i]) for i in range(3)]


def b3_cross(x, y):
    return [b_sub(b_mul(x[1], y[2]), b_mul(y[1], x[2])), b_sub(b_mul(x[2], y[0]), b_mul(y[2], x[0])),
            b_sub(b_mul(x[0], y[1]), b_mul(y[0], x[1]))]


def b3_dot(a, b):
    return b_add(b_add(b_mul(a[0], b[0]), b_mul(a[1], b[1])), b_mul(a[2], b[2]))


def d_cross(x, y):
    return [x[1] * y[2] - y[1] * x[2], x[2] * y[0] - y[2] * x[0], x[0] * y[1] - y[0] * x[1]]


def d_dot(a, b):
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]


def d_sub(a, b):
    return [a[i] - b[i] for i in range(3)]


def _edges(k, p2, p3, q1, q2, q3, z):
    """The factors of axis k's cross product as the kernels pick them (k >= 2)."""
    i = (k - 2) // 3 if k < 11 else k - 11
    j = (k - 2) % 3 if k < 11 else k - 14
    E = ((p2, z), (p3, p2), (z, p3))[min(i, 2)]
    Fj = ((q2, q1), (q3, q2), (q1, q3))[min(j, 2)]
    return E, Fj


def check_pair(P, Q):
    """Every projection's FP64 value inside the double-float interval; returns the axes checked."""
    P = [np.asarray(v, F) for v in P]
    Q = [np.asarray(v, F) for v in Q]
    rel = [[b_rel(V[c], P[0][c]) for c in range(3)] for V in (P[1], P[2], Q[0], Q[1], Q[2])]
    p2, p3, q1, q2, q3 = rel
    zb = ((F(0.0), F(0.0)), F(0.0))
    Z = [zb, zb, zb]
    n1 = b3_cross(p2, b3_sub(p3, p2))
    m1 = b3_cross(b3_sub(q2, q1), b3_sub(q3, q2))
    d = [[float(V[c]) - float(P[0][c]) for c in range(3)] for V in (P[1], P[2], Q[0], Q[1], Q[2])]
    dp2, dp3, dq1, dq2, dq3 = d
    dz = [0.0, 0.0, 0.0]
    dn1 = d_cross(dp2, d_sub(dp3, dp2))
    dm1 = d_cross(d_sub(dq2, dq1), d_sub(dq3, dq2))
    for k in range(17):
        if k == 0:
            ax, dax = n1, dn1
        elif k == 1:
            ax, dax = m1, dm1
        else:
            (ea, eb), (fa, fb) = _edges(k, p2, p3, q1, q2, q3, Z)
            (dea, deb), (dfa, dfb) = _edges(k, dp2, dp3, dq1, dq2, dq3, dz)
            E, Fv = b3_sub(ea, eb), b3_sub(fa, fb)
            dE, dF = d_sub(dea, deb), d_sub(dfa, dfb)
            if k < 11:
                ax, dax = b3_cross(E, Fv), d_cross(dE, dF)
            elif k < 14:
                ax, dax = b3_cross(E, n1), d_cross(dE, dn1)
            else:
                ax, dax = b3_cross(Fv, m1), d_cross(dF, dm1)
        for v3, dv3 in ((p2, dp2), (p3, dp3), (q1, dq1), (q2, dq2), (q3, dq3)):
            (h, l), W = b3_dot(ax, v3)
            v = F(h + l)
            w = mul_ru(F(2.0), add_ru(W, mul_ru(F(2.0 ** -23), abs(v))))
            lo, hi = sub_rd(v, w), add_ru(v, w)
            x = d_dot(dax, dv3)
            assert float(lo) <= x <= float(hi), f"axis {k}: FP64 {x!r} outside [{lo!r}, {hi!r}]"
    return 17


def _pairs(rng, n):
    out = []
    for t in range(n):
        scale = float(2.0 ** rng.integers(-18, 18))
        P = rng.standard_normal((3, 3)) * scale
        kind = t % 3
        if kind == 0:  # crossing or nearby triangles
            Q = P[rng.permutation(3)] + rng.standard_normal((3, 3)) * scale * 10.0 ** rng.uniform(-3, 0)
        elif kind == 1:  # nearly coplanar: both in a plane, B lifted by 1e-7 of the extent
            P[:, 2] *= 1e-6
            Q = P + rng.standard_normal((3, 3)) * scale * 0.3
            Q[:, 2] = P[:, 2].mean() + scale * 1e-7 * rng.standard_normal()
        else:  # exactly coplanar (z = const)
            P[:, 2] = scale
            Q = P + rng.standard_normal((3, 3)) * scale * 0.3
            Q[:, 2] = scale
        out.append((P.astype(np.float32), Q.astype(np.float32)))
    return out


def test_double_float_intervals_hold_the_fp64_values():
    rng = np.random.default_rng(20261204)
    checked = 0
    for P, Q in _pairs(rng, 45):
        checked += check_pair(P, Q)
    assert checked == 45 * 17


def test_rounding_helper_matches_numpy():
    rng = np.random.default_rng(5)
    for _ in range(300):
        a, b = F(rng.standard_normal() * 2.0 ** rng.integers(-30, 30)), F(rng.standard_normal())
        assert _round(_exact(a) + _exact(b), "rn") == F(a + b)
        assert _round(_exact(a) * _exact(b), "rn") == F(a * b)
        up, dn = _round(_exact(a) * _exact(b), "ru"), _round(_exact(a) * _exact(b), "rd")
        assert _exact(dn) <= _exact(a) * _exact(b) <= _exact(up)
        assert up == dn or np.nextafter(dn, _UP) == up


def _edge_pairs(rng):
    """Relative extents at the ends of the pass's range (2^-20: low parts and
    bounds in the float subnormals) and inside it; collinear (zero-area)
    triangles, a shared vertex, coplanar triangles sharing an edge."""
    out = []
    for t in range(48):
        scale = (2.0 ** -20.5, 2.0 ** -20, 2.0 ** 18.5, 1.0, 2.0 ** -10, 2.0 ** 10)[t % 6]
        P = rng.standard_normal((3, 3)) * scale
        form = t % 4
        if form == 0:  # A collinear
            P[2] = P[0] + 0.5 * (P[1] - P[0])
            Q = P[rng.permutation(3)] + rng.standard_normal((3, 3)) * scale * 1e-3
        elif form == 1:  # a shared vertex
            Q = P.copy()
            Q[1:] += rng.standard_normal((2, 3)) * scale
        elif form == 2:  # coplanar, sharing an edge
            P[:, 2] = scale
            Q = P.copy()
            Q[2] = P[2] + rng.standard_normal(3) * scale
            Q[2, 2] = scale
        else:
            Q = P[rng.permutation(3)] + rng.standard_normal((3, 3)) * scale * 1e-3
        P32, Q32 = P.astype(np.float32), Q.astype(np.float32)
        A = np.abs(np.concatenate([P32[1:] - P32[0], Q32 - P32[0]])).max()
        if 2.0 ** -20 <= A <= 2.0 ** 20:  # the pass's range (others go to FP64 whole)
            out.append((P32, Q32))
    return out


def test_double_float_intervals_at_the_range_ends_and_degenerate_triangles():
    pairs = _edge_pairs(np.random.default_rng(99))
    assert len(pairs) >= 40
    for P, Q in pairs:
        check_pair(P, Q)
