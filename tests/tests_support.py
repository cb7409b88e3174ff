"""Seeded input builders shared by the GPU tests."""
import numpy as np

from oibvh_gb300 import meshes as M


def soup(rng, n_tri, scale=0.25):
    base = rng.uniform(0.0, 1.0, size=(n_tri, 1, 3))
    off = rng.uniform(-scale, scale, size=(n_tri, 3, 3))
    xyz = (base + off).reshape(-1, 3).astype(np.float32)
    return M.Mesh(xyz, np.arange(3 * n_tri, dtype=np.uint32).reshape(-1, 3))


def soup_pair(seed):
    rng = np.random.Generator(np.random.PCG64(1000 + seed))
    sizes = [1, 2, 3, 7, 31, 64, 65, 300, 1000, 2049, 4095, 5000]
    na, nb = sizes[seed % len(sizes)], sizes[(seed * 7 + 3) % len(sizes)]
    return [soup(rng, na, 0.3 / max(1.0, na ** 0.33)), soup(rng, nb, 0.3 / max(1.0, nb ** 0.33))]


def mixed_scene(seed):
    rng = np.random.Generator(np.random.PCG64(2000 + seed))
    meshes = []
    n = 4 + seed % 3
    for k in range(n):
        kind = (seed + k) % 3
        if kind == 0:
            m = M.noise_displace(M.icosphere(int(rng.integers(1, 5))), 0.08, seed=int(rng.integers(1 << 30)))
        elif kind == 1:
            m = M.grid_sheet(int(rng.integers(4, 40)), 2.0, 0.2, float(rng.uniform(0.3, 1.0)), origin=(-1, -1, 0))
        else:
            m = soup(rng, int(rng.integers(1, 3000)), 0.05)
            m = M.Mesh((m.xyz * 2 - 1).astype(np.float32), m.tri)
        m = M.rigid_transform(m, M.random_rotation(rng), rng.uniform(-0.5, 0.5, 3))
        meshes.append(m)
    if seed % 2 == 0:
        pairs = None
    else:
        allp = [(i, j) for i in range(n) for j in range(n) if i != j]
        pick = rng.choice(len(allp), size=min(5, len(allp)), replace=False)
        pairs = np.array([allp[i] for i in pick], dtype=np.uint32)
    return meshes, pairs
