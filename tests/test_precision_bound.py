"""The static margin bound of precision mode's first pass, checked on the CPU.

`k_prec_classify` takes a float hit as a hit in FP64 too when every one of
its 17 axes overlaps by more than a bound on the float and FP64 errors:
2^-14 A^3 for the edge x edge axes and the normals, 2^-10 A^4 for the edge x
normal axes, with A the largest relative coordinate (and A in [2^-20, 2^20]).
This restates that rule with numpy's IEEE float32 arithmetic in the
reference's operation order (src/utils/utils.cpp:71-169: relative vertices,
edges, glm cross and dot, min/max, strict comparisons) and checks, on random,
nearly coplanar and rescaled triangle pairs, that no pair the rule calls a hit
is separated by the same formula in float64.
"""
import numpy as np


def _cross(x, y):
    return np.stack([x[:, 1] * y[:, 2] - y[:, 1] * x[:, 2], x[:, 2] * y[:, 0] - y[:, 2] * x[:, 0],
                     x[:, 0] * y[:, 1] - y[:, 0] * x[:, 1]], 1)


def _dot(a, b):
    return (a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1]) + a[:, 2] * b[:, 2]


def _margins(P1, P2, P3, Q1, Q2, Q3):
    """Per axis (reference order) the projections' (mn1, mx1, mn2, mx2), and A."""
    p1 = np.zeros_like(P1)
    p2, p3, q1, q2, q3 = P2 - P1, P3 - P1, Q1 - P1, Q2 - P1, Q3 - P1
    e1, e2, e3 = p2 - p1, p3 - p2, p1 - p3
    f1, f2, f3 = q2 - q1, q3 - q2, q1 - q3
    n1, m1 = _cross(e1, e2), _cross(f1, f2)
    axes = [n1, m1] + [_cross(e, f) for e in (e1, e2, e3) for f in (f1, f2, f3)]
    axes += [_cross(e, n1) for e in (e1, e2, e3)] + [_cross(f, m1) for f in (f1, f2, f3)]
    out = []
    for ax in axes:
        P = np.stack([_dot(ax, p1), _dot(ax, p2), _dot(ax, p3)], 1)
        Q = np.stack([_dot(ax, q1), _dot(ax, q2), _dot(ax, q3)], 1)
        out.append((P.min(1), P.max(1), Q.min(1), Q.max(1)))
    A = np.max(np.abs(np.concatenate([p2, p3, q1, q2, q3], 1)), 1)
    return out, A


def test_robust_float_hits_are_fp64_hits():
    rng = np.random.default_rng(2026)
    robust_total = 0
    for trial in range(30):
        n = 20000
        # the last six trials at the ends of the rule's range [2^-20, 2^20]
        scale = np.float32(2.0 ** (rng.integers(-18, 18) if trial < 24 else (-20.5, 18.5)[trial % 2]))
        P = (rng.standard_normal((n, 3, 3)) * scale).astype(np.float32)
        jitter = rng.standard_normal((n, 3, 3)) * float(scale) * 10.0 ** rng.uniform(-7, 0)
        Q = (P[:, rng.permutation(3)] + jitter).astype(np.float32)
        if trial % 3 == 0:  # nearly coplanar
            P[:, :, 2] = (P[:, :, 2] * np.float32(1e-6)).astype(np.float32)
            Q[:, :, 2] = (Q[:, :, 2] * np.float32(1e-6)).astype(np.float32)
        tri = [P[:, 0], P[:, 1], P[:, 2], Q[:, 0], Q[:, 1], Q[:, 2]]
        m32, A = _margins(*tri)
        m64, _ = _margins(*(x.astype(np.float64) for x in tri))
        A3 = (A * A * A).astype(np.float32)
        B3, B4 = np.float32(2.0 ** -14) * A3, np.float32(2.0 ** -10) * A3 * A
        robust = (A >= 2.0 ** -20) & (A <= 2.0 ** 20)
        hit32, hit64 = np.ones(n, bool), np.ones(n, bool)
        for k in range(17):
            mn1, mx1, mn2, mx2 = m32[k]
            B = B3 if k < 11 else B4
            hit32 &= ~((mn1 > mx2) | (mn2 > mx1))
            robust &= ((mn1 - mx2) < -B) & ((mn2 - mx1) < -B)
            d = m64[k]
            hit64 &= ~((d[0] > d[3]) | (d[2] > d[1]))
        r = hit32 & robust
        robust_total += int(r.sum())
        assert not np.any(r & ~hit64), f"trial {trial}: a robust float hit is separated in FP64"
    assert robust_total > 10000  # the rule decides many hits, so the check is not vacuous
