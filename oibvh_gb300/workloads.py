"""The named synthetic workloads (seeded, deterministic).

plain       two icospheres s=5 (20,480 triangles, 10,242 vertices each),
            radius 1, centres (-0.9,0,0) and (0.9,0,0): build, refit once,
            broad + narrow, sorted pair set.
deforming   two noise-displaced icospheres s=8 (1,310,720 triangles each);
            mesh B gets a seeded random rigid transform placing it so that
            about 1% of its surface lies inside A (the overlapping cap).
            Every frame adds fresh per-vertex Gaussian jitter (sigma 1e-3)
            to the rest positions of both meshes, refits both trees and
            detects.
batched     `n_pairs` independent pairs of noise-displaced icospheres whose
            subdivision is drawn so triangle counts are log-uniform over
            1k..1M; each pair gets a seeded rigid transform that puts
            30..70% of B's surface inside A.
serving     a pool of `n_meshes` noise-displaced icospheres, subdivision drawn
            so triangle counts are log-uniform over 500..2M (s = 3..8, a few
            noise variants per subdivision, each pool entry its own resident
            tree), and a seeded stream of queries (mesh A, mesh B, rigid
            transform of B: random rotation, translation of length
            U(0.3, 1.8) so that most pairs overlap partially).
sheets      `n_pairs` pairs of n x n-quad grid sheets (2n^2 triangles) with a
            sine height field (amplitude 0.1, wavelength U(0.05, 0.5), seeded
            direction and phase). B is the same surface sampled on the grid
            shifted by n - round(0.1 n) columns, so its first 10% of columns
            coincide with A's last ones; odd pairs also lift B by a seeded
            dz in [-1e-7, 1e-7]. Those triangles are coplanar with A's (or
            within 1e-7 of them): the precision stress.

"Overlap fraction" of a pair = fraction of B's surface inside A's ball,
computed from the sphere-cap area: for balls of radii a >= b at distance d
the cut plane lies x = (d^2 + b^2 - a^2) / (2d) from B's centre and the cap
inside A is (b - x) / (2b) of B's area.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import meshes as M


@dataclass
class PairWorkload:
    name: str
    meshes: list                       # rest meshes
    pairs: list                        # (i, j) mesh pairs tested
    jitter_sigma: float = 0.0
    seed: int = 0
    info: dict = field(default_factory=dict)

    def frame_positions(self, frame: int) -> list:
        """Positions of every mesh at `frame` (frame 0 = rest positions)."""
        if frame == 0 or self.jitter_sigma == 0.0:
            return [m.xyz for m in self.meshes]
        return [M.jitter(m.xyz, self.jitter_sigma, self.seed * 1000 + i, frame) for i, m in enumerate(self.meshes)]


def plain() -> PairWorkload:
    a = M.icosphere(5, 1.0, (-0.9, 0.0, 0.0))
    b = M.icosphere(5, 1.0, (0.9, 0.0, 0.0))
    return PairWorkload("plain: 2 icospheres s=5, centres 1.8 apart", [a, b], [(0, 1)])


def _unit_vector(rng: np.random.Generator) -> np.ndarray:
    while True:
        v = rng.uniform(-1.0, 1.0, 3)
        n2 = float(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
        if 1e-6 < n2 <= 1.0:
            return v / math.sqrt(n2)


def distance_for_overlap(a: float, b: float, frac: float) -> float:
    """Centre distance at which `frac` of sphere B (radius b <= a) lies inside ball A."""
    x = b * (1.0 - 2.0 * frac)
    return x + math.sqrt(x * x - b * b + a * a)


def deforming(subdiv: int = 8, seed: int = 2024, overlap: float = 0.01, noise: float = 0.05,
              sigma: float = 1e-3) -> PairWorkload:
    rng = np.random.Generator(np.random.PCG64(seed))
    base = M.icosphere(subdiv)
    a = M.noise_displace(base, noise, seed=seed + 1)
    b0 = M.noise_displace(base, noise, seed=seed + 2)
    R = M.random_rotation(rng)
    d = distance_for_overlap(1.0, 1.0, overlap)
    t = _unit_vector(rng) * d
    b = M.rigid_transform(b0, R, t)
    w = PairWorkload(f"deforming: 2 noise icospheres s={subdiv}, {overlap:.0%} overlap, jitter {sigma:g}",
                     [a, b], [(0, 1)], jitter_sigma=sigma, seed=seed)
    w.info = {"subdiv": subdiv, "triangles_per_mesh": a.n_triangles, "vertices_per_mesh": a.n_vertices,
              "centre_distance": d, "overlap_target": overlap}
    return w


# icosphere subdivision -> triangles: 20 * 4^s (s=3: 1,280 ... s=7: 327,680)
_BATCH_SUBDIVS = (3, 4, 5, 6, 7)


def _subdiv_probs(lo: float = 1e3, hi: float = 1e6, subdivs=_BATCH_SUBDIVS) -> np.ndarray:
    """Probability of each subdivision so that log(T) is uniform over [lo, hi]:
    each s takes the log-mass of the interval around its T (midpoints in log space)."""
    logs = np.array([math.log(20 * 4 ** s) for s in subdivs])
    edges = np.concatenate([[math.log(lo)], (logs[1:] + logs[:-1]) / 2, [math.log(hi)]])
    w = np.clip(np.diff(edges), 0, None)
    return w / w.sum()


@dataclass
class BatchWorkload:
    """Mesh pairs placed by rigid transforms: meshes[2p] = A (identity),
    meshes[2p+1] = B. `rest` are the untransformed meshes and `base[i]` the
    3x4 placement of mesh i (float64); frame f rotates every B about its own
    centre by f * spin_deg degrees around a seeded axis."""

    name: str
    rest: list
    base: list
    pairs: list
    centers: list
    axes: list
    spin_deg: float = 0.5
    info: dict = field(default_factory=dict)

    def matrices(self, frame: int) -> np.ndarray:
        """float32[n_meshes, 12]: row-major 3x4 transforms of every mesh at `frame`."""
        out = np.empty((len(self.rest), 12), dtype=np.float64)
        for i, M in enumerate(self.base):
            if i % 2 == 1 and frame:
                ang = math.radians(self.spin_deg * frame)
                R = _axis_angle(self.axes[i], ang)
                c = self.centers[i]
                # x -> Rf (M x - c) + c, composed in float64
                Rm = R @ M[:, :3]
                t = R @ (M[:, 3] - c) + c
                M = np.concatenate([Rm, t[:, None]], 1)
            out[i] = M.reshape(-1)
        return out.astype(np.float32)

    def positions(self, frame: int, which=None) -> list:
        """Transformed float32 positions of every mesh (or of the meshes listed
        in `which`), computed as the device does:
        x' = ((m0 x + m1 y) + m2 z) + m3 with float32 rounding at each step."""
        mats = self.matrices(frame)
        idx = range(len(self.rest)) if which is None else which
        return [rigid_apply(self.rest[i].xyz, mats[i]) for i in idx]

    def packed_rest_xyzw(self) -> np.ndarray:
        return np.concatenate([np.pad(m.xyz, ((0, 0), (0, 1))) for m in self.rest], 0).astype(np.float32)


def rigid_apply(xyz: np.ndarray, mat12) -> np.ndarray:
    """x' = ((m0 x + m1 y) + m2 z) + m3 per row, float32 rounding at each
    step: the device transform's arithmetic (row-major 3x4 matrix)."""
    M = np.asarray(mat12, dtype=np.float32).reshape(12)
    x, y, z = (np.asarray(xyz, dtype=np.float32)[:, k] for k in range(3))
    rows = []
    for r in range(3):
        a = (M[4 * r] * x + M[4 * r + 1] * y) + M[4 * r + 2] * z
        rows.append((a + M[4 * r + 3]).astype(np.float32))
    return np.stack(rows, 1)


def _axis_angle(axis, ang):
    x, y, z = axis
    c, s = math.cos(ang), math.sin(ang)
    C = 1 - c
    return np.array([[c + x * x * C, x * y * C - z * s, x * z * C + y * s],
                     [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
                     [z * x * C - y * s, z * y * C + x * s, c + z * z * C]], dtype=np.float64)


def batched(n_pairs: int = 512, seed: int = 77, noise: float = 0.05, frac_lo: float = 0.3, frac_hi: float = 0.7,
            subdivs=_BATCH_SUBDIVS, variants: int = 4) -> BatchWorkload:
    """`n_pairs` pairs of noise-displaced icospheres, subdivision drawn so that
    triangle counts are log-uniform over 1k..1M (s = 3..7); B has radius
    U(0.6, 1) and sits where 30..70% of its surface lies inside A.
    (`variants` noise fields per subdivision are generated and reused.)"""
    rng = np.random.Generator(np.random.PCG64(seed))
    probs = _subdiv_probs()
    if tuple(subdivs) != _BATCH_SUBDIVS:
        probs = np.ones(len(subdivs)) / len(subdivs)
    cache = {}

    def mesh(s, k):
        if (s, k) not in cache:
            cache[(s, k)] = noise_displace_mesh(s, noise, seed * 1000 + 10 * s + k)
        return cache[(s, k)]

    rest, base, pairs, centers, axes, fracs = [], [], [], [], [], []
    for p in range(n_pairs):
        sa, sb = (int(x) for x in rng.choice(subdivs, size=2, p=probs))
        ka, kb = (int(x) for x in rng.integers(0, variants, 2))
        rb = float(rng.uniform(0.6, 1.0))
        frac = float(rng.uniform(frac_lo, frac_hi))
        a = mesh(sa, ka)
        b0 = mesh(sb, kb)
        b = M.Mesh((b0.xyz.astype(np.float64) * rb).astype(np.float32), b0.tri)
        d = distance_for_overlap(1.0, rb, frac)
        R = M.random_rotation(rng)
        t = _unit_vector(rng) * d
        rest += [a, b]
        base += [np.concatenate([np.eye(3), np.zeros((3, 1))], 1), np.concatenate([R, t[:, None]], 1)]
        centers += [np.zeros(3), t.copy()]
        axes += [np.array([0.0, 0.0, 1.0]), _unit_vector(rng)]
        pairs.append((2 * p, 2 * p + 1))
        fracs.append(frac)
    tri = np.array([m.n_triangles for m in rest])
    w = BatchWorkload(f"batched: {n_pairs} pairs of noise icospheres, T log-uniform 1k-1M, 30-70% overlap",
                      rest, base, pairs, centers, axes)
    w.info = {"n_pairs": n_pairs, "meshes": len(rest), "triangles_total": int(tri.sum()),
              "triangles_min": int(tri.min()), "triangles_max": int(tri.max()),
              "vertices_total": int(sum(m.n_vertices for m in rest)), "overlap_mean": float(np.mean(fracs))}
    return w


_ICO_CACHE = {}


def noise_displace_mesh(subdiv: int, amplitude: float, seed: int) -> "M.Mesh":
    if subdiv not in _ICO_CACHE:
        _ICO_CACHE[subdiv] = M.icosphere(subdiv)
    return M.noise_displace(_ICO_CACHE[subdiv], amplitude, seed=seed)


def sheet_pair_meshes(n: int, wavelength: float, theta: float, phase: float, dz: float,
                      amplitude: float = 0.1, overlap: float = 0.1):
    """Sheets A and B of one pair (float32 positions, uint32 faces).

    Vertex (i, j) of a sheet whose first column is c0 sits at
    x = (c0 + i) / n, y = j / n (exact in float32), height
    z = amplitude * sin(2 pi (x cos(theta) + y sin(theta)) / wavelength + phase)
    computed in float64 and rounded once; B's heights get `dz` added before
    rounding. Faces split each quad (v00, v10, v11), (v00, v11, v01), row-major.
    """
    shift = n - int(round(overlap * n))

    def sheet(c0: int, lift: float) -> "M.Mesh":
        cols = np.arange(n + 1, dtype=np.float64) + c0
        rows = np.arange(n + 1, dtype=np.float64)
        x, y = np.meshgrid(cols / n, rows / n, indexing="xy")
        x = x.reshape(-1)
        y = y.reshape(-1)
        arg = 2.0 * np.pi * (x * math.cos(theta) + y * math.sin(theta)) / wavelength + phase
        z = amplitude * M._sin_poly(arg) + lift
        xyz = np.stack([x, y, z], 1).astype(np.float32)
        q = np.arange(n, dtype=np.int64)
        qx, qy = np.meshgrid(q, q, indexing="xy")
        v00 = (qy * (n + 1) + qx).reshape(-1)
        v10, v01 = v00 + 1, v00 + (n + 1)
        v11 = v01 + 1
        tri = np.empty((2 * n * n, 3), dtype=np.int64)
        tri[0::2] = np.stack([v00, v10, v11], 1)
        tri[1::2] = np.stack([v00, v11, v01], 1)
        return M.Mesh(xyz, tri.astype(np.uint32))

    return sheet(0, 0.0), sheet(shift, dz)


@dataclass
class SheetWorkload:
    name: str
    meshes: list
    pairs: list
    info: dict = field(default_factory=dict)


def sheets(n_pairs: int = 64, n: int = 256, seed: int = 4242, overlap: float = 0.1) -> SheetWorkload:
    rng = np.random.Generator(np.random.PCG64(seed))
    meshes, pairs, lifts = [], [], []
    for p in range(n_pairs):
        wl = float(rng.uniform(0.05, 0.5))
        theta = float(rng.uniform(0.0, 2.0 * math.pi))
        phase = float(rng.uniform(0.0, 2.0 * math.pi))
        dz = 0.0 if p % 2 == 0 else float(rng.uniform(-1e-7, 1e-7))
        a, b = sheet_pair_meshes(n, wl, theta, phase, dz, overlap=overlap)
        meshes += [a, b]
        pairs.append((2 * p, 2 * p + 1))
        lifts.append(dz)
    w = SheetWorkload(f"sheets: {n_pairs} pairs of {n}x{n}-quad sine sheets, {overlap:.0%} coplanar or within 1e-7",
                      meshes, pairs)
    w.info = {"n_pairs": n_pairs, "quads": n, "triangles_per_sheet": 2 * n * n, "vertices_per_sheet": (n + 1) ** 2,
              "overlap_columns": int(round(overlap * n)), "lifted_pairs": int(sum(1 for d in lifts if d != 0.0)),
              "triangles_total": 2 * n * n * 2 * n_pairs}
    return w


_SERVE_SUBDIVS = (3, 4, 5, 6, 7, 8)


@dataclass
class ServingWorkload:
    name: str
    meshes: list        # pool entry -> mesh (entries share the variant meshes)
    variant_of: list    # pool entry -> (subdivision, variant)
    info: dict = field(default_factory=dict)

    def queries(self, n: int, seed: int = 1):
        """n queries: (mesh A, mesh B, float32[12] row-major 3x4 transform of B)."""
        from . import meshes as M

        rng = np.random.Generator(np.random.PCG64(seed))
        ab = rng.integers(0, len(self.meshes), size=(n, 2))
        mats = np.empty((n, 12), dtype=np.float32)
        for k in range(n):
            R = M.random_rotation(rng)
            t = _unit_vector(rng) * float(rng.uniform(0.3, 1.8))
            mats[k] = np.concatenate([R, t[:, None]], 1).reshape(12)
        return ab.astype(np.uint32), mats


def serving(n_meshes: int = 2000, seed: int = 5150, variants: int = 3, noise: float = 0.05,
            lo: float = 500.0, hi: float = 2e6) -> ServingWorkload:
    rng = np.random.Generator(np.random.PCG64(seed))
    probs = _subdiv_probs(lo, hi, _SERVE_SUBDIVS)
    cache = {}
    meshes, var = [], []
    for _ in range(n_meshes):
        s_ = int(rng.choice(_SERVE_SUBDIVS, p=probs))
        k = int(rng.integers(0, variants))
        if (s_, k) not in cache:
            cache[(s_, k)] = noise_displace_mesh(s_, noise, seed * 1000 + 10 * s_ + k)
        meshes.append(cache[(s_, k)])
        var.append((s_, k))
    tri = np.array([m.n_triangles for m in meshes], dtype=np.int64)
    w = ServingWorkload(f"serving: pool of {n_meshes} noise icospheres, T log-uniform 500-2M", meshes, var)
    w.info = {"pool_meshes": n_meshes, "triangles_total": int(tri.sum()), "triangles_min": int(tri.min()),
              "triangles_max": int(tri.max()), "triangles_mean": float(tri.mean()),
              "distinct_host_meshes": len(cache)}
    return w
