"""Precision mode on the GPU: the FP64-filtered triangle test against the
all-FP64 oracle, and the float mode against the reference's float test.

The FP64 oracle (oracle_tri_intersect_f64) evaluates the reference's 17-axis
test (src/utils/utils.cpp:97-169) in double over the same float inputs, with
the same exact-AABB candidate set. The filtered mode must reproduce its pair
set with zero mismatches; the float mode must stay bit-exact with the
reference's float test; and the device's count of candidates where the two
answers differ must equal the size of the symmetric difference of the two
oracle pair sets.
"""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from oracle.oracle import Port, sort_pairs
from tests_support import near_degenerate_pair

pytestmark = pytest.mark.gpu


def _oracle_sets(meshes, pairs):
    p = Port()
    for m in meshes:
        p.add_mesh(m.xyz, m.tri)
    pr = None if pairs is None else np.asarray(pairs, dtype=np.uint32)
    h32, c32 = p.detect(pr)
    h64, _ = p.detect(pr, fp64=True)
    return sort_pairs(h32), sort_pairs(h64), c32


def _scene(meshes, pairs):
    from oibvh_gb300 import OibvhTree, Scene

    trees = [OibvhTree(m) for m in meshes]
    for t in trees:
        t.build()
    sc = Scene()
    for t in trees:
        sc.addOibvhTree(t)
    if pairs is not None:
        sc.set_pairs(pairs)
    return sc, trees


def _run(sc, mode, entry=0):
    from oibvh_gb300 import DeviceType, _native as N

    sc.set_precision(mode)
    sc.detectCollision(DeviceType.GPU0, entry, 1)
    return sc.int_tri_pairs(), sc.stats()


def _sym(a, b):
    sa = set(map(tuple, a.tolist()))
    sb = set(map(tuple, b.tolist()))
    return len(sa ^ sb)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_near_degenerate_pairs(gpu, seed):
    from oibvh_gb300 import _native as N

    meshes = list(near_degenerate_pair(seed))
    want32, want64, cands = _oracle_sets(meshes, None)
    assert _sym(want32, want64) > 0  # the input does reach the float/FP64 boundary
    sc, _ = _scene(meshes, None)
    got32, st32 = _run(sc, N.PRECISION_FP32)
    assert np.array_equal(got32, want32)
    got64, st64 = _run(sc, N.PRECISION_FP64_FILTERED)
    assert np.array_equal(got64, want64), f"{_sym(got64, want64)} mismatches against the FP64 oracle"
    assert st64["candidates"] == cands
    assert st64["fp32_disagreements"] == _sym(want32, want64)
    # the FP64 pass takes only what the bounded and double-float passes left undecided
    assert 0 <= st64["fp64_candidates"] <= st64["bounded_candidates"] <= cands
    assert st64["bounded_candidates"] > 0
    assert st32["fp64_axes"] == 0 and st32["bounded_candidates"] == 0


def test_sheets_small(gpu):
    from oibvh_gb300 import _native as N
    from oibvh_gb300 import workloads as W

    w = W.sheets(8, 64, seed=11)
    want32, want64, _ = _oracle_sets(w.meshes, w.pairs)
    sc, _ = _scene(w.meshes, w.pairs)
    got32, _ = _run(sc, N.PRECISION_FP32, entry=2)
    assert np.array_equal(got32, want32)
    got64, st = _run(sc, N.PRECISION_FP64_FILTERED, entry=2)
    assert np.array_equal(got64, want64)
    assert st["fp32_disagreements"] == _sym(want32, want64)


def test_precision_frame_graph_and_split_phases(gpu):
    """The captured frame and the split broad/narrow calls honour the mode."""
    from oibvh_gb300 import DeviceType, _native as N

    meshes = list(near_degenerate_pair(7, n_tri=800))
    _, want64, _ = _oracle_sets(meshes, None)
    sc, trees = _scene(meshes, None)
    sc.set_precision(N.PRECISION_FP64_FILTERED)
    sc.capture_frame(0, 1, True)
    for _ in range(2):
        sc.launch_frame()
        sc.finish_frame()
        assert np.array_equal(sc.int_tri_pairs(), want64)
    sc.broad(DeviceType.GPU0, 0, 1)
    sc.narrow()
    assert np.array_equal(sc.int_tri_pairs(), want64)
    assert sc.precision() == N.PRECISION_FP64_FILTERED


def test_sheets_full_size_zero_mismatches(gpu):
    """64 pairs of 256x256-quad sheets: every pair's filtered set equals the
    FP64 oracle's; float/FP64 disagreements are counted per pair."""
    from oibvh_gb300 import _native as N
    from oibvh_gb300 import workloads as W

    w = W.sheets(64, 256)
    sc, _ = _scene(w.meshes, w.pairs)
    got64, st = _run(sc, N.PRECISION_FP64_FILTERED, entry=4)

    def one(pair):
        a, b = pair
        p = Port()
        p.add_mesh(w.meshes[a].xyz, w.meshes[a].tri)
        p.add_mesh(w.meshes[b].xyz, w.meshes[b].tri)
        h64, _ = p.detect(fp64=True)
        h64 = h64.copy()
        h64[:, 0] = a
        h64[:, 1] = b
        return h64

    with ThreadPoolExecutor(8) as ex:
        parts = list(ex.map(one, w.pairs))
    want64 = sort_pairs(np.concatenate(parts, 0))
    assert np.array_equal(got64, want64), f"{_sym(got64, want64)} mismatches against the FP64 oracle"
    # the double-float pass decides these (sheets within 1e-7 of each other) without FP64
    assert st["bounded_candidates"] >= st["fp64_candidates"]


def _coplanar_soup(seed, n_tri=600):
    """Two soups of triangles in the plane z = 0.5 (exactly representable):
    their normal axes project both sets to exactly the same value, so neither
    the float bounds nor the double-float pass can decide them; FP64 does."""
    from oibvh_gb300.meshes import Mesh

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(2):
        c = rng.uniform(0.0, 1.0, (n_tri, 1, 2))
        v = c + rng.uniform(-0.03, 0.03, (n_tri, 3, 2))
        xyz = np.concatenate([v.reshape(-1, 2), np.full((3 * n_tri, 1), 0.5)], 1).astype(np.float32)
        out.append(Mesh(xyz, np.arange(3 * n_tri, dtype=np.uint32).reshape(-1, 3)))
    return out


@pytest.mark.parametrize("seed", [0, 1])
def test_coplanar_soups_take_the_fp64_pass(gpu, seed):
    from oibvh_gb300 import _native as N

    meshes = _coplanar_soup(seed)
    _, want64, cands = _oracle_sets(meshes, None)
    sc, _ = _scene(meshes, None)
    got64, st = _run(sc, N.PRECISION_FP64_FILTERED)
    assert np.array_equal(got64, want64), f"{_sym(got64, want64)} mismatches against the FP64 oracle"
    assert st["candidates"] == cands
    assert st["fp64_candidates"] > 0 and st["fp64_axes"] > 0  # the FP64 pass ran


def test_precision_argument_checks(gpu):
    from oibvh_gb300 import OibvhError, Scene

    sc = Scene()
    with pytest.raises(OibvhError):
        sc.set_precision(5)
