"""Seeded synthetic meshes for the collision workloads.

The reference loads ``bunny.obj`` through assimp (src/main.cpp:127,
src/utils/model.cpp:40-82); that file is not shipped with it, so every
workload here is generated: subdivided icospheres, radially displaced by a
gradient noise, grid sheets with a sine height field, seeded rigid transforms
and per-frame Gaussian jitter.

Determinism: the geometry is computed in float64 with element-wise numpy
operations only (add, multiply, divide, sqrt, floor: all correctly rounded,
so identical on x86-64 and aarch64) and rounded once to float32.
``mesh_digest`` gives a SHA-256 over the exact bytes, which the golden
fixtures store next to the pair sets they pin.

Layout: positions are ``float32[V, 3]`` (xyz), faces ``uint32[T, 3]``.
"""
from __future__ import annotations

import hashlib
from dataclasses import dataclass

import numpy as np

__all__ = [
    "Mesh",
    "icosphere",
    "grid_sheet",
    "perlin3",
    "noise_displace",
    "random_rotation",
    "rigid_transform",
    "jitter",
    "mesh_digest",
    "load_obj",
    "save_obj",
]


@dataclass
class Mesh:
    """Positions (float32[V,3]) and faces (uint32[T,3]) of one triangle mesh."""

    xyz: np.ndarray
    tri: np.ndarray

    @property
    def n_vertices(self) -> int:
        return int(self.xyz.shape[0])

    @property
    def n_triangles(self) -> int:
        return int(self.tri.shape[0])

    def copy(self) -> "Mesh":
        return Mesh(self.xyz.copy(), self.tri.copy())


def _unit(v: np.ndarray) -> np.ndarray:
    n = np.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
    return v / n[:, None]


def _icosphere_unit(subdiv: int) -> tuple[np.ndarray, np.ndarray]:
    t = (1.0 + np.sqrt(5.0)) / 2.0
    v = np.array(
        [
            [-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
            [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
            [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1],
        ],
        dtype=np.float64,
    )
    f = np.array(
        [
            [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
            [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
            [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
            [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1],
        ],
        dtype=np.int64,
    )
    v = _unit(v)
    for _ in range(subdiv):
        nv = v.shape[0]
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        edges = np.stack([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)], 1).reshape(-1, 2)
        lo = np.minimum(edges[:, 0], edges[:, 1])
        hi = np.maximum(edges[:, 0], edges[:, 1])
        key = lo * nv + hi
        uniq, inv = np.unique(key, return_inverse=True)
        mid = _unit((v[uniq // nv] + v[uniq % nv]) * 0.5)
        v = np.concatenate([v, mid], 0)
        m = (inv + nv).reshape(-1, 3)
        ab, bc, ca = m[:, 0], m[:, 1], m[:, 2]
        # the four children of face i become faces 4i..4i+3, so faces that are
        # close in index are close in space (the usual in-place subdivision order)
        f = np.stack(
            [
                np.stack([a, ab, ca], 1),
                np.stack([b, bc, ab], 1),
                np.stack([c, ca, bc], 1),
                np.stack([ab, bc, ca], 1),
            ],
            1,
        ).reshape(-1, 3)
    return v, f


def icosphere(subdiv: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)) -> Mesh:
    """Subdivided icosahedron: 20*4^s triangles, 10*4^s+2 vertices."""
    v, f = _icosphere_unit(int(subdiv))
    xyz = v * float(radius) + np.asarray(center, dtype=np.float64)[None, :]
    return Mesh(xyz.astype(np.float32), f.astype(np.uint32))


def grid_sheet(n: int, size: float = 1.0, amplitude: float = 0.0, wavelength: float = 1.0,
               origin=(0.0, 0.0, 0.0)) -> Mesh:
    """n x n quads (2n^2 triangles, (n+1)^2 vertices) in the xy plane with
    height z = amplitude * sin(2 pi x / wavelength) * cos(2 pi y / wavelength).

    The sine is evaluated with a 13-term Taylor polynomial after exact range
    reduction to [-pi, pi], so the heights do not depend on the platform's libm.
    """
    g = np.arange(n + 1, dtype=np.float64) * (float(size) / n)
    x, y = np.meshgrid(g, g, indexing="xy")
    x = x.reshape(-1)
    y = y.reshape(-1)
    z = float(amplitude) * _sin_poly(2.0 * np.pi * x / wavelength) * _sin_poly(2.0 * np.pi * y / wavelength + np.pi / 2)
    xyz = np.stack([x, y, z], 1) + np.asarray(origin, dtype=np.float64)[None, :]
    i = np.arange(n, dtype=np.int64)
    qx, qy = np.meshgrid(i, i, indexing="xy")
    v00 = (qy * (n + 1) + qx).reshape(-1)
    v10 = v00 + 1
    v01 = v00 + (n + 1)
    v11 = v01 + 1
    tri = np.concatenate([np.stack([v00, v10, v11], 1), np.stack([v00, v11, v01], 1)], 0)
    order = np.argsort(np.concatenate([np.arange(n * n) * 2, np.arange(n * n) * 2 + 1]), kind="stable")
    tri = tri[order]
    return Mesh(xyz.astype(np.float32), tri.astype(np.uint32))


def _sin_poly(a: np.ndarray) -> np.ndarray:
    two_pi = 2.0 * np.pi
    r = a - two_pi * np.floor(a / two_pi + 0.5)
    r2 = r * r
    term = r.copy()
    acc = r.copy()
    for k in range(1, 13):
        term = -term * r2 / ((2 * k) * (2 * k + 1))
        acc = acc + term
    return acc


def _perm_table(seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    p = rng.permutation(256).astype(np.int64)
    return np.concatenate([p, p])


def _fade(t: np.ndarray) -> np.ndarray:
    return t * t * t * (t * (t * 6.0 - 15.0) + 10.0)


def _grad(h: np.ndarray, x: np.ndarray, y: np.ndarray, z: np.ndarray) -> np.ndarray:
    h = h & 15
    u = np.where(h < 8, x, y)
    v = np.where(h < 4, y, np.where((h == 12) | (h == 14), x, z))
    return np.where((h & 1) == 0, u, -u) + np.where((h & 2) == 0, v, -v)


def perlin3(p: np.ndarray, seed: int) -> np.ndarray:
    """Gradient noise in 3D following Perlin's published improved-noise method
    (quintic fade, 12 edge gradients, lattice hashing through a permutation),
    with a seeded permutation. Input float64[N,3], output float64[N] in ~[-1,1]."""
    perm = _perm_table(seed)
    fl = np.floor(p)
    ci = fl.astype(np.int64) & 255
    f = p - fl
    X, Y, Z = ci[:, 0], ci[:, 1], ci[:, 2]
    x, y, z = f[:, 0], f[:, 1], f[:, 2]
    u, v, w = _fade(x), _fade(y), _fade(z)
    A = perm[X] + Y
    AA = perm[A] + Z
    AB = perm[A + 1] + Z
    B = perm[X + 1] + Y
    BA = perm[B] + Z
    BB = perm[B + 1] + Z

    def lerp(t, a, b):
        return a + t * (b - a)

    return lerp(
        w,
        lerp(v, lerp(u, _grad(perm[AA], x, y, z), _grad(perm[BA], x - 1, y, z)),
             lerp(u, _grad(perm[AB], x, y - 1, z), _grad(perm[BB], x - 1, y - 1, z))),
        lerp(v, lerp(u, _grad(perm[AA + 1], x, y, z - 1), _grad(perm[BA + 1], x - 1, y, z - 1)),
             lerp(u, _grad(perm[AB + 1], x, y - 1, z - 1), _grad(perm[BB + 1], x - 1, y - 1, z - 1))),
    )


def noise_displace(mesh: Mesh, amplitude: float, seed: int, frequency: float = 4.0,
                   center=(0.0, 0.0, 0.0)) -> Mesh:
    """Move every vertex radially (about `center`) by amplitude * noise(frequency * x)."""
    c = np.asarray(center, dtype=np.float64)[None, :]
    p = mesh.xyz.astype(np.float64) - c
    r = np.sqrt(p[:, 0] * p[:, 0] + p[:, 1] * p[:, 1] + p[:, 2] * p[:, 2])
    d = np.where(r[:, None] > 0, p / np.where(r > 0, r, 1.0)[:, None], 0.0)
    n = perlin3(p * float(frequency) + 17.0, seed)
    q = c + d * (r + float(amplitude) * n)[:, None]
    return Mesh(q.astype(np.float32), mesh.tri.copy())


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniform random rotation matrix from a unit quaternion drawn by
    Marsaglia's rejection method (uniforms and sqrt only)."""
    while True:
        x1, y1 = rng.uniform(-1.0, 1.0, 2)
        s1 = x1 * x1 + y1 * y1
        if s1 < 1.0:
            break
    while True:
        x2, y2 = rng.uniform(-1.0, 1.0, 2)
        s2 = x2 * x2 + y2 * y2
        if s2 < 1.0:
            break
    k = np.sqrt((1.0 - s1) / s2)
    w, x, y, z = x1, y1, x2 * k, y2 * k
    return np.array(
        [
            [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
            [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
            [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
        ],
        dtype=np.float64,
    )


def rigid_transform(mesh: Mesh, rotation: np.ndarray, translation, pivot=(0.0, 0.0, 0.0)) -> Mesh:
    """x' = R (x - pivot) + pivot + t, evaluated in float64, rounded to float32."""
    pv = np.asarray(pivot, dtype=np.float64)[None, :]
    p = mesh.xyz.astype(np.float64) - pv
    R = np.asarray(rotation, dtype=np.float64)
    q = np.empty_like(p)
    for r in range(3):
        q[:, r] = (p[:, 0] * R[r, 0] + p[:, 1] * R[r, 1]) + p[:, 2] * R[r, 2]
    q = q + pv + np.asarray(translation, dtype=np.float64)[None, :]
    return Mesh(q.astype(np.float32), mesh.tri.copy())


def jitter(xyz: np.ndarray, sigma: float, seed: int, frame: int) -> np.ndarray:
    """Per-vertex Gaussian jitter N(0, sigma^2) for one frame, seeded by (seed, frame)."""
    rng = np.random.Generator(np.random.PCG64([int(seed), int(frame)]))
    return (xyz.astype(np.float64) + rng.standard_normal(xyz.shape) * float(sigma)).astype(np.float32)


def mesh_digest(*arrays: np.ndarray) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def load_obj(path: str) -> Mesh:
    """Minimal Wavefront OBJ reader for the collision path: `v x y z [w]`
    positions and `f` faces (`i`, `i/t`, `i//n`, `i/t/n`, 1-based or negative
    relative indices); polygons are split into fans (v0, vi, vi+1), the
    triangulation the reference's loader asks assimp for (aiProcess_Triangulate,
    src/utils/model.cpp:49-51). Normals, texture coordinates, groups and
    materials are ignored: collision reads positions and index triples only.
    Positions are parsed as float64 and rounded once to float32."""
    xyz: list = []
    tri: list = []
    with open(path, "r", encoding="utf-8", errors="replace") as fh:
        for ln, line in enumerate(fh, 1):
            parts = line.split("#", 1)[0].split()
            if not parts:
                continue
            if parts[0] == "v":
                if len(parts) < 4:
                    raise ValueError(f"{path}:{ln}: vertex needs three coordinates")
                xyz.append((float(parts[1]), float(parts[2]), float(parts[3])))
            elif parts[0] == "f":
                idx = []
                for tok in parts[1:]:
                    k = int(tok.split("/", 1)[0])
                    k = k - 1 if k > 0 else len(xyz) + k
                    if not 0 <= k < len(xyz):
                        raise ValueError(f"{path}:{ln}: face refers to vertex {tok} of {len(xyz)}")
                    idx.append(k)
                if len(idx) < 3:
                    raise ValueError(f"{path}:{ln}: a face needs three vertices")
                for i in range(1, len(idx) - 1):
                    tri.append((idx[0], idx[i], idx[i + 1]))
    if not tri:
        raise ValueError(f"{path}: no faces")
    return Mesh(np.asarray(xyz, dtype=np.float64).astype(np.float32), np.asarray(tri, dtype=np.uint32))


def save_obj(mesh: Mesh, path: str) -> None:
    """Write positions and triangles as OBJ (positions with float32 round-trip precision)."""
    with open(path, "w", encoding="utf-8") as fh:
        # 9 significant digits identify a float32 exactly
        for x, y, z in mesh.xyz.astype(np.float32).astype(np.float64).tolist():
            fh.write(f"v {x:.9g} {y:.9g} {z:.9g}\n")
        for a, b, c in (mesh.tri.astype(np.int64) + 1).tolist():
            fh.write(f"f {a} {b} {c}\n")
