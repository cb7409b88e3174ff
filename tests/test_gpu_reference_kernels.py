"""The tree layout and the pair sets against the reference's OWN GPU kernels
(src/cuda/oibvh.cu, src/cuda/collide.cu compiled unmodified for sm_103a,
driven headless by oracle/ref_gpu_harness.cu), run on the same inputs:

* Morton order (sorted faces) bit-exact on config 1 (two icospheres s=5);
* every node box bit-exact after the reference's build and refit, on meshes
  whose construction schedule runs full blocks only (power-of-two triangle
  counts: the harness refuses the others before launching, because the
  reference's construction kernels reach __syncthreads after an early return);
* the broad phase's candidate count equal, and the pair sets equal on generic
  inputs; on the coplanar sheets of config 4 the reference's GPU narrow phase
  (compiled with nvcc's default FMA contraction) may disagree with its own CPU
  arithmetic, which this library follows: the disagreements are counted.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle.oracle import Port, RefGPU, sort_pairs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref(gpu):
    if not RefGPU.available():
        pytest.skip("reference GPU kernels not built (oracle/build_ref.sh)")
    return RefGPU


def _pow2_meshes():
    from oibvh_gb300 import meshes as M
    from oibvh_gb300 import workloads as W
    from tests_support import soup

    rng = np.random.Generator(np.random.PCG64(77))
    return [M.grid_sheet(32, 1.0, 0.1, 0.4), soup(rng, 1024, 0.05), W.sheets(1, 256).meshes[0],
            M.grid_sheet(64, 2.0, 0.3, 0.7, origin=(-1.0, -1.0, 0.0))]


def test_morton_order_config1(ref):
    """Sorted faces of the reference's GPU build (its leaf-box + Morton kernel
    and thrust's two stable sorts) equal this library's, on config 1; the
    harness refuses the construction there (partial blocks)."""
    from oibvh_gb300 import OibvhTree

    g = load_golden("config1")
    for m in g["meshes"]:
        rt = ref.Tree(m.xyz, m.tri)
        st, _ = rt.build(construct=True)
        assert st == ref.UNSAFE_SCHEDULE
        st, _ = rt.build(construct=False)
        assert st == ref.OK
        t = OibvhTree(m)
        t.build()
        f, _ = t.sorted_faces()
        assert np.array_equal(rt.sorted_faces(), f)


def test_tree_build_and_refit_bit_exact(ref):
    from oibvh_gb300 import OibvhTree

    rng = np.random.default_rng(5)
    for m in _pow2_meshes():
        rt = ref.Tree(m.xyz, m.tri)
        st, _ = rt.build()
        assert st == ref.OK, m.n_triangles
        t = OibvhTree(m)
        t.build()
        f, _ = t.sorted_faces()
        assert np.array_equal(rt.sorted_faces(), f)
        assert np.array_equal(rt.boxes().view(np.uint32), t.aabb_tree().view(np.uint32))
        moved = (m.xyz + rng.normal(scale=1e-3, size=m.xyz.shape)).astype(np.float32)
        st, _ = rt.refit(moved)
        assert st == ref.OK
        t.refit(moved)
        assert np.array_equal(rt.boxes().view(np.uint32), t.aabb_tree().view(np.uint32))


def _ours(meshes, entry=4, expand=3):
    from oibvh_gb300 import DeviceType, OibvhTree, Scene

    trees = [OibvhTree(m) for m in meshes]
    for t in trees:
        t.build()
    sc = Scene()
    for t in trees:
        sc.addOibvhTree(t)
    sc.detectCollision(DeviceType.GPU0, entry, expand)
    return sc.int_tri_pairs(), sc.candidate_count(), [t.sorted_faces()[1] for t in trees]


def _ref_pairs(ref, meshes, perms, entry=4, expand=3):
    rts = [ref.Tree(m.xyz, m.tri) for m in meshes]
    for rt in rts:
        assert rt.build()[0] == ref.OK
    n, hits, ncand, _ = ref.detect(rts, entry, expand)
    assert n >= 0, n
    hits = hits.copy()
    hits[:, 2] = perms[0][hits[:, 2]]  # Morton order -> original face index
    hits[:, 3] = perms[1][hits[:, 3]]
    return sort_pairs(hits), ncand


def test_detect_generic_pair_sets_equal(ref):
    """Two overlapping soups of 1,024 triangles and two crossing sheets: the
    reference's GPU pair set and candidate count equal this library's."""
    from oibvh_gb300 import meshes as M
    from tests_support import soup

    rng = np.random.Generator(np.random.PCG64(91))
    cases = [[soup(rng, 1024, 0.05), soup(rng, 1024, 0.05)],
             [M.grid_sheet(32, 1.0, 0.2, 0.3),
              M.rigid_transform(M.grid_sheet(32, 1.0, 0.2, 0.5), M.random_rotation(rng), (0.1, 0.05, 0.0))]]
    for meshes in cases:
        ours, oc, perms = _ours(meshes)
        got, rc = _ref_pairs(ref, meshes, perms)
        assert rc == oc
        assert ours.shape[0] > 0
        assert np.array_equal(got, ours)


def test_detect_config4_sheets_counts_and_disagreements(ref):
    """Config 4's sheets (131,072 triangles each, 10 % coplanar or within
    1e-7): equal candidate counts (the broad phase is exact min/max work), and
    the reference's GPU narrow phase (nvcc's default FMA contraction) differs
    from the reference's CPU arithmetic (this library's) on at most 1 % of the
    hits: near-degenerate pairs. The count is printed as a finding."""
    from oibvh_gb300 import workloads as W

    w = W.sheets(2, 256)
    total, hits = 0, 0
    for a, b in w.pairs:
        meshes = [w.meshes[a], w.meshes[b]]
        ours, oc, perms = _ours(meshes)
        got, rc = _ref_pairs(ref, meshes, perms)
        assert rc == oc
        key = lambda h: set(map(tuple, h[:, 2:].tolist()))
        total += len(key(got) ^ key(ours))
        hits += ours.shape[0]
    assert hits > 0 and total <= hits // 100
    print(f"reference GPU narrow phase vs the reference CPU arithmetic: {total} differing pairs of {hits} hits")
