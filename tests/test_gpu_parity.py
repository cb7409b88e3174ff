"""CUDA path vs the reference's pair sets (golden fixtures) and vs the oracle port.

Bit-exact: the colliding-pair set, the candidate count, the Morton order and
every node box of the tree (integer / min-max work, no tolerance)."""
import numpy as np
import pytest

from cases import CASES
from conftest import load_golden
from oracle.oracle import Port, sort_pairs

pytestmark = pytest.mark.gpu


def run_gpu(meshes, pairs, frames, entry, expand):
    from oibvh_gb300 import DeviceType, OibvhTree, Scene

    trees = [OibvhTree(m) for m in meshes]
    for t in trees:
        t.build()
    sc = Scene()
    for t in trees:
        sc.addOibvhTree(t)
    if pairs is not None:
        sc.set_pairs(pairs)
    out = []
    sc.detectCollision(DeviceType.GPU0, entry, expand)
    out.append((sc.int_tri_pairs(), sc.candidate_count()))
    for fr in frames:
        for t, xyz in zip(trees, fr):
            t.refit(xyz)
        sc.detectCollision(DeviceType.GPU0, entry, expand)
        out.append((sc.int_tri_pairs(), sc.candidate_count()))
    return out


@pytest.mark.parametrize("entry,expand", [(0, 1), (4, 3), (2, 2), (30, 1)])
@pytest.mark.parametrize("name", sorted(CASES))
def test_golden_pair_sets(gpu, name, entry, expand):
    g = load_golden(name)
    res = run_gpu(g["meshes"], g["pairs"], g["frames"], entry, expand)
    for f, (hits, ncand) in enumerate(res):
        assert hits.shape == g["hits"][f].shape, f"frame {f}: {hits.shape[0]} hits, expected {g['hits'][f].shape[0]}"
        assert np.array_equal(hits, g["hits"][f]), f"frame {f}"
        assert ncand == g["candidates"][f], f"frame {f}"


@pytest.mark.parametrize("name", ["config1", "noise_spheres", "soups", "three_bodies"])
def test_tree_layout_bit_exact(gpu, name):
    from oibvh_gb300 import OibvhTree

    g = load_golden(name)
    for m in g["meshes"]:
        t = OibvhTree(m)
        t.build()
        aabbs, st, perm = Port.oibvh_build(m.xyz, m.tri)
        f, p = t.sorted_faces()
        assert np.array_equal(p, perm)
        assert np.array_equal(f, st)
        got = t.aabb_tree()
        assert got.shape == aabbs.shape
        assert np.array_equal(got.view(np.uint32), aabbs.view(np.uint32))
        assert t.getPrimCount() == m.n_triangles
        assert t.getDepth() == int(np.floor(np.log2(aabbs.shape[0])))


def test_refit_layout_bit_exact(gpu):
    from oibvh_gb300 import OibvhTree

    g = load_golden("deforming")
    m = g["meshes"][0]
    t = OibvhTree(m)
    t.build()
    st, _ = t.sorted_faces()
    for fr in g["frames"]:
        t.refit(fr[0])
        want = Port.oibvh_refit(fr[0], st)
        assert np.array_equal(t.aabb_tree().view(np.uint32), want.view(np.uint32))


def _oracle_pairs(meshes, pairs=None):
    p = Port()
    for m in meshes:
        p.add_mesh(m.xyz, m.tri)
    h, c = p.detect(pairs)
    return sort_pairs(h), c


@pytest.mark.parametrize("seed", range(12))
def test_random_soups_vs_oracle(gpu, seed):
    from tests_support import soup_pair

    meshes = soup_pair(seed)
    want, wc = _oracle_pairs(meshes)
    got = run_gpu(meshes, None, [], seed % 5, 1 + seed % 3)[0]
    assert np.array_equal(got[0], want) and got[1] == wc


@pytest.mark.parametrize("seed", range(4))
def test_random_scenes_vs_oracle(gpu, seed):
    """4-6 meshes of mixed kinds, all pairs or a random subset of pairs."""
    from tests_support import mixed_scene

    meshes, pairs = mixed_scene(seed)
    want, wc = _oracle_pairs(meshes, pairs)
    got = run_gpu(meshes, pairs, [], 3, 2)[0]
    assert np.array_equal(got[0], want) and got[1] == wc


def test_deforming_s8_frames_vs_oracle(gpu):
    """The deforming workload at full size (1,310,720 triangles per mesh): the
    rest pose and ten jittered frames, each refit and detected."""
    from oibvh_gb300 import workloads as W

    w = W.deforming()
    frames = [w.frame_positions(f) for f in range(1, 11)]
    res = run_gpu(w.meshes, None, frames, 4, 3)
    p = Port()
    for m in w.meshes:
        p.add_mesh(m.xyz, m.tri)
    for f in range(len(frames) + 1):
        if f:
            for i, xyz in enumerate(frames[f - 1]):
                p.set_positions(i, xyz)
        want, wc = p.detect()
        assert np.array_equal(res[f][0], sort_pairs(want)), f"frame {f}"
        assert res[f][1] == wc


def test_scene_refit_one_launch_bit_exact(gpu):
    """oibvh_scene_refit: every tree refit in one launch equals the oracle's refit."""
    from oibvh_gb300 import DeviceType, OibvhTree, Scene

    g = load_golden("three_bodies")
    trees = [OibvhTree(m) for m in g["meshes"]]
    for t in trees:
        t.build()
    sc = Scene()
    for t in trees:
        sc.addOibvhTree(t)
    rng = np.random.default_rng(0)
    moved = [(m.xyz + rng.normal(scale=1e-3, size=m.xyz.shape)).astype(np.float32) for m in g["meshes"]]
    for t, x in zip(trees, moved):
        t.set_positions(x)
    sc.refit()
    for t, x in zip(trees, moved):
        st, _ = t.sorted_faces()
        assert np.array_equal(t.aabb_tree().view(np.uint32), Port.oibvh_refit(x, st).view(np.uint32))
    sc.detectCollision(DeviceType.GPU0, 4, 1)
    want, wc = _oracle_pairs([type(g["meshes"][0])(x, m.tri) for x, m in zip(moved, g["meshes"])])
    assert np.array_equal(sc.int_tri_pairs(), want) and sc.candidate_count() == wc


def test_wide_morton_keys_order_and_pair_set(gpu):
    """63-bit keys (21 bits per axis): the leaf order is the restated one, a
    scene build agrees with per-tree builds, and the pair set is unchanged."""
    from oibvh_gb300 import DeviceType, OibvhTree, Scene
    from oibvh_gb300 import meshes as M
    from oibvh_gb300 import workloads as W
    from tests_support import morton63_order

    meshes = [W.noise_displace_mesh(5, 0.05, 11), W.noise_displace_mesh(4, 0.05, 12)]
    meshes[1] = M.rigid_transform(meshes[1], np.eye(3), (0.8, 0.2, 0.1))
    trees = [OibvhTree(m) for m in meshes]
    for t, m in zip(trees, meshes):
        t.set_morton_bits(63)
        assert t.morton_bits() == 63
        t.build()
        _, perm = t.sorted_faces()
        assert np.array_equal(perm, morton63_order(m.xyz, m.tri))
    sc = Scene()
    for t in trees:
        sc.addOibvhTree(t)
    sc.detectCollision(DeviceType.GPU0, 4, 3)
    port = Port()
    for m in meshes:
        port.add_mesh(m.xyz, m.tri)
    want, wc = port.detect()
    assert np.array_equal(sc.int_tri_pairs(), sort_pairs(want)) and want.shape[0] > 0
    assert sc.candidate_count() == wc
    # the same trees built together
    trees2 = [OibvhTree(m) for m in meshes]
    sc2 = Scene()
    for t in trees2:
        t.set_morton_bits(63)
        sc2.addOibvhTree(t)
    sc2.build()
    for t, t2 in zip(trees, trees2):
        assert np.array_equal(t.sorted_faces()[1], t2.sorted_faces()[1])
        assert np.array_equal(t.aabb_tree().view(np.uint32), t2.aabb_tree().view(np.uint32))


def test_top_walk_handoff_widths_keep_every_pair(gpu):
    """The single-CTA top walk hands its front to the walkers once it is wider
    than the handoff width; its front buffer holds 8,192 pairs and a wider
    level spills to the walkers' list. With a handoff above 2,048 a level of
    at most `handoff` pairs can have more than 8,192 children, so the front
    handed over must be appended after the spilled pairs, not written over
    them. Two nearly coincident spheres give fronts of 5,098 and then 10,253
    pairs from start level 4: handoffs of 6,000 and 8,000 take that path."""
    from oibvh_gb300 import DeviceType, OibvhTree, Scene
    from oibvh_gb300 import meshes as M
    from tests_support import bvtt_front_widths

    a = M.icosphere(5, 1.0, (0.0, 0.0, 0.0))
    b = M.icosphere(5, 1.0, (0.01, 0.0, 0.0))
    widths = bvtt_front_widths(a, b, 4)
    spills = [h for h in (6000, 8000) if any(w0 <= h and w1 > 8192 for w0, w1 in zip(widths, widths[1:]))]
    assert spills == [6000, 8000], widths  # the case reaches the spill for both widths
    want, wc = _oracle_pairs([a, b])
    trees = [OibvhTree(m) for m in (a, b)]
    for t in trees:
        t.build()
    sc = Scene()
    for t in trees:
        sc.addOibvhTree(t)
    for handoff in (32, 2048, 4096, 6000, 8000, 8192):
        sc.set_tuning(start_pairs_log2=8, handoff=handoff)  # one pair: start level 4
        sc.detectCollision(DeviceType.GPU0, 0, 1)
        got = sc.int_tri_pairs()
        assert got.shape == want.shape, f"handoff {handoff}: {got.shape[0]} pairs, expected {want.shape[0]}"
        assert np.array_equal(got, want), f"handoff {handoff}"
        assert sc.candidate_count() == wc, f"handoff {handoff}"
