"""The C restatement (oracle port) against the golden fixtures that the
reference's own CPU path produced (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from cases import CASES
from conftest import load_golden
from oracle.oracle import Port, Reference, sort_pairs


@pytest.mark.parametrize("name", sorted(CASES))
def test_port_matches_reference_fixture(name):
    g = load_golden(name)
    port = Port()
    for m in g["meshes"]:
        port.add_mesh(m.xyz, m.tri)
    hits, ncand = port.detect(g["pairs"])
    assert np.array_equal(sort_pairs(hits), g["hits"][0])
    assert ncand == g["candidates"][0]
    for f, fr in enumerate(g["frames"], start=1):
        for i, xyz in enumerate(fr):
            port.set_positions(i, xyz)
        hits, ncand = port.detect(g["pairs"])
        assert np.array_equal(sort_pairs(hits), g["hits"][f]), f"frame {f}"
        assert ncand == g["candidates"][f]


@pytest.mark.skipif(not Reference.available(), reason="reference CPU path not built here (oracle/_ref)")
@pytest.mark.parametrize("name", sorted(CASES))
def test_fixture_is_current(name):
    """Where the reference checkout exists, the fixtures are what it computes."""
    g = load_golden(name)
    ref = Reference()
    for m in g["meshes"]:
        ref.add_mesh(m.xyz, m.tri)
    hits, ncand = ref.detect(g["pairs"])
    assert np.array_equal(sort_pairs(hits), g["hits"][0])
    assert ncand == g["candidates"][0]


@pytest.mark.skipif(not Reference.available(), reason="reference CPU path not built here (oracle/_ref)")
def test_port_sat_matches_reference_random():
    rng = np.random.default_rng(123)
    tri = (rng.normal(size=(20000, 6, 3)) * 0.4).astype(np.float32)
    # also near-degenerate: second triangle coplanar with the first
    tri[::4, 3:, 2] = tri[::4, :3, 2].mean(axis=1, keepdims=True)
    for t in tri:
        assert Port.tri_intersect(*t) == Reference.tri_intersect(*t)


@pytest.mark.skipif(not Reference.available(), reason="reference CPU path not built here (oracle/_ref)")
def test_port_leaf_boxes_match_reference():
    g = load_golden("noise_spheres")
    port, ref = Port(), Reference()
    for m in g["meshes"]:
        port.add_mesh(m.xyz, m.tri)
        ref.add_mesh(m.xyz, m.tri)
    for i in range(len(g["meshes"])):
        assert np.array_equal(port.leaf_boxes(i).view(np.uint32), ref.leaf_boxes(i).view(np.uint32))


def test_fp64_oracle_agrees_away_from_degeneracy():
    """FP64 SAT equals FP32 SAT on well-separated random triangles."""
    rng = np.random.default_rng(5)
    agree = 0
    for _ in range(3000):
        t = (rng.normal(size=(6, 3)) * 0.5).astype(np.float32)
        agree += Port.tri_intersect(*t) == Port.tri_intersect(*t, fp64=True)
    assert agree >= 2990
