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


def test_obj_round_trip_is_exact(tmp_path):
    m = M.noise_displace(M.icosphere(3), 0.05, seed=3)
    p = tmp_path / "sphere.obj"
    M.save_obj(m, str(p))
    r = M.load_obj(str(p))
    assert np.array_equal(r.xyz.view(np.uint32), m.xyz.view(np.uint32))
    assert np.array_equal(r.tri, m.tri)


def test_obj_reader_forms(tmp_path):
    p = tmp_path / "forms.obj"
    p.write_text(
        "# a quad, a pentagon and a triangle with relative indices\n"
        "o first\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvn 0 0 1\nvt 0 0\n"
        "f 1/1/1 2/1/1 3/1/1 4/1/1\n"
        "g second\nv 0 0 1\nv 1 0 1\nv 2 1 1\nv 1 2 1\nv 0 1 1  # trailing comment\n"
        "f 5//1 6//1 7//1 8//1 9//1\n"
        "f -3 -2 -1\n")
    m = M.load_obj(str(p))
    assert m.n_vertices == 9
    assert m.tri.tolist() == [[0, 1, 2], [0, 2, 3], [4, 5, 6], [4, 6, 7], [4, 7, 8], [6, 7, 8]]
    assert m.xyz.dtype == np.float32


def test_obj_reader_rejects_bad_faces(tmp_path):
    p = tmp_path / "bad.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nf 1 2 3\n")
    with pytest.raises(ValueError):
        M.load_obj(str(p))
