"""Synthetic mesh generators: counts, topology, determinism."""
import numpy as np
import pytest

from oibvh_gb300 import meshes as M


@pytest.mark.parametrize("s", [0, 1, 2, 3, 5])
def test_icosphere_counts_and_closed(s):
    m = M.icosphere(s)
    assert m.n_triangles == 20 * 4**s and m.n_vertices == 10 * 4**s + 2
    e = np.sort(np.concatenate([m.tri[:, [0, 1]], m.tri[:, [1, 2]], m.tri[:, [2, 0]]]), axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    assert np.all(counts == 2)  # closed 2-manifold
    r = np.linalg.norm(m.xyz.astype(np.float64), axis=1)
    assert np.allclose(r, 1.0, atol=1e-6)


def test_grid_sheet_counts():
    g = M.grid_sheet(8, 1.0, 0.1, 0.5)
    assert g.n_triangles == 2 * 64 and g.n_vertices == 81
    assert g.tri.max() < g.n_vertices


def test_generators_deterministic():
    a = M.noise_displace(M.icosphere(3), 0.05, seed=4)
    b = M.noise_displace(M.icosphere(3), 0.05, seed=4)
    assert M.mesh_digest(a.xyz, a.tri) == M.mesh_digest(b.xyz, b.tri)
    rng1, rng2 = np.random.default_rng(1), np.random.default_rng(1)
    assert np.array_equal(M.random_rotation(rng1), M.random_rotation(rng2))
    R = M.random_rotation(np.random.default_rng(9))
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-12) and abs(np.linalg.det(R) - 1) < 1e-12


def test_perlin_range():
    p = np.random.default_rng(0).uniform(-10, 10, size=(5000, 3))
    n = M.perlin3(p, seed=3)
    assert np.all(np.abs(n) <= 1.01) and n.std() > 0.1
