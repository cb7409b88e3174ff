"""Definitions of the golden parity cases (shared by make_golden.py and the tests).

Each case is a list of meshes (xyz float32[V,3], tri uint32[T,3]), an optional
list of mesh pairs (None = every i<j, the reference's Scene default), and
optional extra frames of positions (refit inputs).
"""
from __future__ import annotations

import numpy as np

from oibvh_gb300 import meshes as M


def _soup(rng, n_tri, lo=0.0, hi=1.0, scale=0.3):
    """n_tri independent random triangles: a random corner in [lo, hi)^3 plus small edges."""
    base = rng.uniform(lo, hi, size=(n_tri, 1, 3))
    off = rng.uniform(-scale, scale, size=(n_tri, 3, 3))
    xyz = (base + off).reshape(-1, 3).astype(np.float32)
    tri = np.arange(3 * n_tri, dtype=np.uint32).reshape(-1, 3)
    return M.Mesh(xyz, tri)


def case_config1():
    """Two icospheres s=5 (20,480 triangles, 10,242 vertices), radius 1, centres 1.8 apart on x."""
    a = M.icosphere(5, 1.0, (-0.9, 0.0, 0.0))
    b = M.icosphere(5, 1.0, (0.9, 0.0, 0.0))
    return dict(meshes=[a, b], pairs=None, frames=None)


def case_noise_spheres():
    """Noise-displaced icospheres s=3, the second rotated and shifted so they interpenetrate."""
    rng = np.random.Generator(np.random.PCG64(7))
    a = M.noise_displace(M.icosphere(3), 0.05, seed=11)
    b0 = M.noise_displace(M.icosphere(3), 0.05, seed=12)
    b = M.rigid_transform(b0, M.random_rotation(rng), (0.8, 0.3, -0.2))
    return dict(meshes=[a, b], pairs=None, frames=None)


def case_soups():
    """Random triangle soups of awkward sizes: 1, 2, 3, 5, 17 and 100 triangles."""
    rng = np.random.Generator(np.random.PCG64(3))
    meshes = [_soup(rng, n) for n in (1, 2, 3, 5, 17, 100)]
    return dict(meshes=meshes, pairs=None, frames=None)


def case_coplanar_sheets():
    """Two flat 16x16 sheets in the same plane, the second shifted by a third of a cell
    in x and y: every overlap is coplanar (strict '>' separation decides)."""
    a = M.grid_sheet(16, 1.0, 0.0, 1.0)
    b = M.grid_sheet(16, 1.0, 0.0, 1.0, origin=(1.0 / 48.0, 1.0 / 48.0, 0.0))
    return dict(meshes=[a, b], pairs=None, frames=None)


def case_touching():
    """Tetrahedra touching at a shared vertex, along a shared edge, on a shared face,
    and one at a distance of one float32 ulp."""
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float32)
    t = np.array([[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]], dtype=np.uint32)
    tet = M.Mesh(v, t)
    vertex = M.Mesh(np.array([[1, 0, 0], [2, 0, 0], [1, 1, 0], [1, 0, 1]], dtype=np.float32), t.copy())
    edge = M.Mesh(np.array([[0, 0, 0], [1, 0, 0], [0.5, -1, 0], [0.5, -0.5, -1]], dtype=np.float32), t.copy())
    face = M.Mesh(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.3, 0.3, -1]], dtype=np.float32), t.copy())
    gap = np.nextafter(np.float32(1.0), np.float32(2.0))
    ulp = M.Mesh(np.array([[gap, 0, 0], [2, 0, 0], [gap, 1, 0], [gap, 0, 1]], dtype=np.float32), t.copy())
    return dict(meshes=[tet, vertex, edge, face, ulp], pairs=[(0, 1), (0, 2), (0, 3), (0, 4)], frames=None)


def case_identical():
    """A mesh tested against an exact copy of itself: every triangle touches itself and
    its neighbours."""
    a = M.noise_displace(M.icosphere(2), 0.1, seed=5)
    return dict(meshes=[a, a.copy()], pairs=None, frames=None)


def case_three_bodies():
    """Three meshes of different sizes, all pairs (the reference Scene's i<j loop)."""
    a = M.icosphere(3, 1.0, (0.0, 0.0, 0.0))
    b = M.icosphere(2, 0.7, (1.2, 0.1, 0.0))
    c = M.grid_sheet(20, 2.5, 0.1, 0.7, origin=(-1.0, -1.0, 0.05))
    return dict(meshes=[a, b, c], pairs=None, frames=None)


def case_deforming():
    """Noise spheres s=4 with a rigid offset, then three frames of Gaussian jitter
    (sigma 1e-3) applied to both meshes: refit-only frames."""
    rng = np.random.Generator(np.random.PCG64(21))
    a = M.noise_displace(M.icosphere(4), 0.05, seed=31)
    b = M.rigid_transform(M.noise_displace(M.icosphere(4), 0.05, seed=32), M.random_rotation(rng), (1.7, 0.2, 0.1))
    frames = []
    for f in range(3):
        frames.append([M.jitter(a.xyz, 1e-3, 100, f), M.jitter(b.xyz, 1e-3, 200, f)])
    return dict(meshes=[a, b], pairs=None, frames=frames)


CASES = {
    "config1": case_config1,
    "noise_spheres": case_noise_spheres,
    "soups": case_soups,
    "coplanar_sheets": case_coplanar_sheets,
    "touching": case_touching,
    "identical": case_identical,
    "three_bodies": case_three_bodies,
    "deforming": case_deforming,
}

# Cases whose inputs are regenerated from the generators (checked by digest)
# instead of being stored in the fixture.
REGENERATED = {"config1"}
