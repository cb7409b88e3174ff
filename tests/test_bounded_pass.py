"""The bounded float pass's decisions (project6_bounded in k_prec_settle and
in k_prec_classify's recheck of the separating axis), checked on the CPU.

The pass carries a bound e on the error of every float quantity of the
reference's 17-axis test (src/utils/utils.cpp:71-169: relative vertices,
edges, glm cross and dot products, each operation rounded once): a relative
vertex errs by at most u|x|, a difference by ea + eb + u|c|, a product by
|a| eb + |b| ea + ea eb + u|c| + 2^-149, u = 2^-24. An axis separates in
every arithmetic when a margin (mn1 - mx2 or mn2 - mx1) exceeds tau = 2
(max projection error of A + that of B), and overlaps in every arithmetic
when both margins are below -tau. This replays that arithmetic in numpy
float32 (correctly rounded, one rounding per operation; the device may fuse
some of the bound's multiply-adds, which the factor 2 covers) and checks on
random, nearly and exactly coplanar triangle pairs, rescaled across the
pass's range [2^-20, 2^20] and to its ends, that every axis the bounds decide
is decided the same way by the FP64 formula.
"""
import numpy as np

F = np.float32
U = F(2.0 ** -24)
ETA = F(2.0 ** -149)


def _err_sub(c, ea, eb):
    return F(ea + eb) + U * np.abs(c)


def _err_mul(a, b, c, ea, eb):
    return F(F(F(np.abs(a) * eb + np.abs(b) * ea) + ea * eb) + U * np.abs(c)) + ETA


def _esub(a, b):
    c = a[0] - b[0]
    return c, _err_sub(c, a[1], b[1])


def _ecross(x, y):
    (xv, xe), (yv, ye) = x, y
    out_v, out_e = np.empty_like(xv), np.empty_like(xv)
    for r, (i, j) in enumerate(((1, 2), (2, 0), (0, 1))):
        m1 = xv[:, i] * yv[:, j]
        m2 = yv[:, i] * xv[:, j]
        c = m1 - m2
        out_v[:, r] = c
        out_e[:, r] = _err_sub(c, _err_mul(xv[:, i], yv[:, j], m1, xe[:, i], ye[:, j]),
                               _err_mul(yv[:, i], xv[:, j], m2, ye[:, i], xe[:, j]))
    return out_v, out_e


def _edot(a, p):
    (av, ae), (pv, pe) = a, p
    t = [av[:, c] * pv[:, c] for c in range(3)]
    s = t[0] + t[1]
    r = s + t[2]
    e = [_err_mul(av[:, c], pv[:, c], t[c], ae[:, c], pe[:, c]) for c in range(3)]
    return r, _err_sub(r, _err_sub(s, e[0], e[1]), e[2])


def _d_cross(x, y):
    return np.stack([x[:, 1] * y[:, 2] - y[:, 1] * x[:, 2], x[:, 2] * y[:, 0] - y[:, 2] * x[:, 0],
                     x[:, 0] * y[:, 1] - y[:, 0] * x[:, 1]], 1)


def _d_dot(a, b):
    return (a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1]) + a[:, 2] * b[:, 2]


def _axes(p2, p3, q1, q2, q3, p1, sub, cross):
    e1, e2, e3 = sub(p2, p1), sub(p3, p2), sub(p1, p3)
    f1, f2, f3 = sub(q2, q1), sub(q3, q2), sub(q1, q3)
    n1, m1 = cross(e1, e2), cross(f1, f2)
    ax = [n1, m1] + [cross(e, f) for e in (e1, e2, e3) for f in (f1, f2, f3)]
    return ax + [cross(e, n1) for e in (e1, e2, e3)] + [cross(f, m1) for f in (f1, f2, f3)]


def _decisions(P1, P2, P3, Q1, Q2, Q3):
    """Per axis: +1 separated in every arithmetic, -1 overlapping in every arithmetic, 0 undecided;
    and the FP64 formula's separation."""
    rel = [V - P1 for V in (P2, P3, Q1, Q2, Q3)]
    A = np.max(np.abs(np.concatenate(rel, 1)), 1)
    ok = (A >= 2.0 ** -20) & (A <= 2.0 ** 20)
    ev = [(v, U * np.abs(v)) for v in rel]
    z = (np.zeros_like(P1), np.zeros_like(P1))
    axes = _axes(*ev, z, _esub, _ecross)
    dv = [V.astype(np.float64) - P1.astype(np.float64) for V in (P2, P3, Q1, Q2, Q3)]
    daxes = _axes(*dv, np.zeros_like(dv[0]), lambda a, b: a - b, _d_cross)
    dec, sep64 = [], []
    for ax, dax in zip(axes, daxes):
        pr = [_edot(ax, v) for v in ev]
        P = [(F(0.0) * pr[0][0], F(0.0) * pr[0][1])] + pr[:2]
        Q = pr[2:]
        mx1, mn1 = np.maximum(np.maximum(P[0][0], P[1][0]), P[2][0]), np.minimum(np.minimum(P[0][0], P[1][0]), P[2][0])
        mx2, mn2 = np.maximum(np.maximum(Q[0][0], Q[1][0]), Q[2][0]), np.minimum(np.minimum(Q[0][0], Q[1][0]), Q[2][0])
        tau = F(2.0) * (np.maximum(np.maximum(P[0][1], P[1][1]), P[2][1]) +
                        np.maximum(np.maximum(Q[0][1], Q[1][1]), Q[2][1]))
        d1, d2 = mn1 - mx2, mn2 - mx1
        d = np.where((d1 > tau) | (d2 > tau), 1, np.where((d1 < -tau) & (d2 < -tau), -1, 0))
        dec.append(np.where(ok, d, 0))
        dP = [np.zeros(len(P1))] + [_d_dot(dax, v) for v in dv[:2]]
        dQ = [_d_dot(dax, v) for v in dv[2:]]
        sep64.append((np.minimum(np.minimum(*dP[:2]), dP[2]) > np.maximum(np.maximum(*dQ[:2]), dQ[2])) |
                     (np.minimum(np.minimum(*dQ[:2]), dQ[2]) > np.maximum(np.maximum(*dP[:2]), dP[2])))
    return np.stack(dec, 1), np.stack(sep64, 1)


def test_bounded_decisions_agree_with_fp64():
    rng = np.random.default_rng(1204)
    decided_sep = decided_overlap = 0
    for trial in range(24):
        n = 20000
        # the last six trials at the ends of the range (2^-20: bounds in the float subnormals)
        scale = np.float32(2.0 ** (rng.integers(-18, 18) if trial < 18 else (-20.5, 18.5)[trial % 2]))
        P = (rng.standard_normal((n, 3, 3)) * scale).astype(np.float32)
        jitter = rng.standard_normal((n, 3, 3)) * float(scale) * 10.0 ** rng.uniform(-7, 0)
        Q = (P[:, rng.permutation(3)] + jitter).astype(np.float32)
        if trial % 3 == 0:  # nearly coplanar
            P[:, :, 2] = (P[:, :, 2] * np.float32(1e-6)).astype(np.float32)
            Q[:, :, 2] = (Q[:, :, 2] * np.float32(1e-6)).astype(np.float32)
        elif trial % 3 == 1:  # exactly coplanar
            P[:, :, 2] = scale
            Q[:, :, 2] = scale
        with np.errstate(over="ignore", under="ignore", invalid="ignore"):
            dec, sep64 = _decisions(P[:, 0], P[:, 1], P[:, 2], Q[:, 0], Q[:, 1], Q[:, 2])
        assert not np.any((dec == 1) & ~sep64), f"trial {trial}: a bounded separation FP64 does not make"
        assert not np.any((dec == -1) & sep64), f"trial {trial}: a bounded overlap FP64 separates"
        decided_sep += int((dec == 1).sum())
        decided_overlap += int((dec == -1).sum())
    assert decided_sep > 100000 and decided_overlap > 100000  # the bounds decide many axes either way
