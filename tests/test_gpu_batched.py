"""Batched path on the GPU: one-launch-per-stage scene build, device rigid
transforms, many pairs per detect, the captured frame graph and the autotuner,
each checked bit-exact against the oracle port."""
import numpy as np
import pytest

from oracle.oracle import Port, sort_pairs

pytestmark = pytest.mark.gpu


def _workload(n_pairs=10, subdivs=(2, 3, 4), seed=5):
    from oibvh_gb300 import workloads as W

    return W.batched(n_pairs, seed=seed, subdivs=subdivs, variants=2)


def _oracle(meshes_xyz, tris, pairs):
    p = Port()
    for x, t in zip(meshes_xyz, tris):
        p.add_mesh(x, t)
    h, c = p.detect(np.asarray(pairs, dtype=np.uint32))
    return sort_pairs(h), c


def _scene_from(w, build_with_scene=True):
    from oibvh_gb300 import OibvhTree, Scene

    trees = [OibvhTree(m) for m in w.rest]
    sc = Scene()
    for t in trees:
        sc.addOibvhTree(t)
    if build_with_scene:
        sc.build()
    else:
        for t in trees:
            t.build()
    sc.set_pairs(w.pairs)
    return sc, trees


def test_scene_build_equals_per_tree_build(gpu):
    w = _workload(12, subdivs=(1, 2, 3, 4))
    sc, trees = _scene_from(w)
    for t, m in zip(trees, w.rest):
        aabbs, st, perm = Port.oibvh_build(m.xyz, m.tri)
        f, p = t.sorted_faces()
        assert np.array_equal(p, perm) and np.array_equal(f, st)
        assert np.array_equal(t.aabb_tree().view(np.uint32), aabbs.view(np.uint32))


def test_transform_refit_detect_vs_oracle(gpu):
    import torch

    from oibvh_gb300 import DeviceType

    w = _workload(10)
    sc, trees = _scene_from(w)
    rest = torch.from_numpy(w.packed_rest_xyzw()).cuda()
    for frame in (0, 3):
        mats = torch.from_numpy(w.matrices(frame)).cuda()
        sc.transform(rest.data_ptr(), mats.data_ptr())
        sc.refit()
        sc.detectCollision(DeviceType.GPU0, 0, 1)
        pos = w.positions(frame)
        # transform arithmetic is the documented float32 formula: leaf boxes match bit for bit
        for t, x in zip(trees[:4], pos[:4]):
            st, _ = t.sorted_faces()
            assert np.array_equal(t.aabb_tree().view(np.uint32), Port.oibvh_refit(x, st).view(np.uint32))
        want, wc = _oracle(pos, [m.tri for m in w.rest], w.pairs)
        assert np.array_equal(sc.int_tri_pairs(), want), f"frame {frame}"
        assert sc.candidate_count() == wc


def test_captured_frame_graph_vs_oracle(gpu):
    import torch

    w = _workload(8, seed=9)
    sc, trees = _scene_from(w)
    rest = torch.from_numpy(w.packed_rest_xyzw()).cuda()
    mats = torch.from_numpy(w.matrices(0)).cuda()
    sc.capture_frame(0, 1, True, rest.data_ptr(), mats.data_ptr())
    for frame in (1, 2, 5):
        mats.copy_(torch.from_numpy(w.matrices(frame)))
        sc.launch_frame()
        sc.finish_frame()
        want, wc = _oracle(w.positions(frame), [m.tri for m in w.rest], w.pairs)
        assert np.array_equal(sc.int_tri_pairs(), want), f"frame {frame}"
        assert sc.candidate_count() == wc
    # the captured walk rounds cover these frames: none was redone synchronously
    assert sc.stats()["frame_redos"] == 0
    # the same frame stage by stage (per-stage times): the same pair set
    mats.copy_(torch.from_numpy(w.matrices(6)))
    prof = sc.profile_frame()
    want, wc = _oracle(w.positions(6), [m.tri for m in w.rest], w.pairs)
    assert np.array_equal(sc.int_tri_pairs(), want) and sc.candidate_count() == wc
    assert prof["walk_rounds"] >= 3 and prof["kernels"] == 4 + prof["walk_rounds"]
    for k in ("transform_ms", "refit_ms", "start_ms", "walk_ms"):
        assert prof[k] > 0.0, k
    assert prof["narrow_ms"] >= 0.0


def test_frame_graph_recovers_from_small_queues(gpu):
    """A frame whose queues are too small is redone synchronously, never truncated."""
    import torch

    w = _workload(6, seed=11)
    sc, trees = _scene_from(w)
    rest = torch.from_numpy(w.packed_rest_xyzw()).cuda()
    mats = torch.from_numpy(w.matrices(0)).cuda()
    sc.capture_frame(0, 1, True, rest.data_ptr(), mats.data_ptr())
    sc.set_queue_capacity(front=16, hits=8)  # invalidates the captured buffers: re-capture on launch
    mats.copy_(torch.from_numpy(w.matrices(4)))
    sc.launch_frame()
    sc.finish_frame()
    want, _ = _oracle(w.positions(4), [m.tri for m in w.rest], w.pairs)
    assert np.array_equal(sc.int_tri_pairs(), want)


def test_autotune_keeps_the_pair_set(gpu):
    from oibvh_gb300 import DeviceType

    w = _workload(10, seed=13)
    sc, trees = _scene_from(w, build_with_scene=False)
    for t, x in zip(trees, w.positions(0)):
        t.refit(x)
    sc.detectCollision(DeviceType.GPU0, 0, 1)
    before = sc.int_tri_pairs()
    chosen = sc.autotune(0, 2)
    assert chosen["handoff"] in (512, 2048, 8192) and chosen["walk_front"] in (64, 128, 256, 512)
    assert chosen["descend_ratio"] in (4, 16, 64, 1 << 30)
    sc.detectCollision(DeviceType.GPU0, 0, 1)
    assert np.array_equal(sc.int_tri_pairs(), before)
    want, _ = _oracle(w.positions(0), [m.tri for m in w.rest], w.pairs)
    assert np.array_equal(before, want)


def test_walker_queue_capacity_keeps_the_pair_set(gpu):
    """Every walker queue capacity (32 runs as the 64-entry minimum) gives the
    oracle's pair set; small queues spill to the next round instead."""
    from oibvh_gb300 import DeviceType, OibvhError

    w = _workload(8, seed=17)
    sc, trees = _scene_from(w, build_with_scene=False)
    for t, x in zip(trees, w.positions(0)):
        t.refit(x)
    want, wc = _oracle(w.positions(0), [m.tri for m in w.rest], w.pairs)
    for cap in (32, 64, 256, 512):
        sc.set_tuning(walk_front=cap)
        assert sc.tuning()["walk_front"] == cap
        sc.detectCollision(DeviceType.GPU0, 0, 1)
        assert np.array_equal(sc.int_tri_pairs(), want), cap
        assert sc.candidate_count() == wc
    with pytest.raises(OibvhError):
        sc.set_tuning(walk_front=48)


def test_descend_ratios_keep_the_pair_set(gpu):
    """However the traversal chooses the side to descend (both sides always,
    the larger box only, or both while the boxes are within a ratio), the pair
    set and the candidate count are the oracle's."""
    from oibvh_gb300 import DeviceType, OibvhError

    w = _workload(8, seed=19, subdivs=(1, 3, 5))
    sc, trees = _scene_from(w, build_with_scene=False)
    for t, x in zip(trees, w.positions(0)):
        t.refit(x)
    want, wc = _oracle(w.positions(0), [m.tri for m in w.rest], w.pairs)
    for r in (1, 2, 16, 64, 1 << 30):
        sc.set_tuning(descend_ratio=r)
        assert sc.tuning()["descend_ratio"] == r
        for entry in (0, 4):
            sc.detectCollision(DeviceType.GPU0, entry, 1)
            assert np.array_equal(sc.int_tri_pairs(), want), (r, entry)
            assert sc.candidate_count() == wc
    with pytest.raises(OibvhError):
        sc.set_tuning(descend_ratio=(1 << 30) + 1)


def test_claim_thresholds_keep_the_pair_set(gpu):
    """Walkers that claim work-list items dynamically (from 1 item per warp on)
    or take static interleaved shares (a threshold above any list) find the
    oracle's pair set and candidate count, in direct detects and in frames."""
    import torch

    from oibvh_gb300 import DeviceType, OibvhError

    w = _workload(12, seed=23, subdivs=(2, 4, 5))
    sc, trees = _scene_from(w)
    rest = torch.from_numpy(w.packed_rest_xyzw()).cuda()
    mats = torch.from_numpy(w.matrices(2)).cuda()
    want, wc = _oracle(w.positions(2), [m.tri for m in w.rest], w.pairs)
    for c in (1, 4, 32, 1 << 20):
        for start in (12, 20):
            sc.set_tuning(claim_min=c, start_pairs_log2=start, handoff=512)
            assert sc.tuning()["claim_min"] == c
            sc.capture_frame(4, 3, True, rest.data_ptr(), mats.data_ptr())
            sc.launch_frame()
            sc.finish_frame()
            assert np.array_equal(sc.int_tri_pairs(), want), (c, start)
            assert sc.candidate_count() == wc
            sc.detectCollision(DeviceType.GPU0, 0, 1)
            assert np.array_equal(sc.int_tri_pairs(), want), (c, start)
    with pytest.raises(OibvhError):
        sc.set_tuning(claim_min=(1 << 20) + 1)


def test_refit_level_group_depths_agree(gpu):
    """The scene refit with level groups of 9, 10 and 11 levels per CTA (two
    climbing stages for the deep tree) writes the oracle's boxes bit for bit."""
    import torch

    from oibvh_gb300 import OibvhTree, Scene
    from oibvh_gb300 import workloads as W

    meshes = [W.noise_displace_mesh(7, 0.05, 3), W.noise_displace_mesh(2, 0.05, 4),
              W.noise_displace_mesh(5, 0.05, 5)]
    trees = [OibvhTree(m) for m in meshes]
    sc = Scene()
    for t in trees:
        sc.addOibvhTree(t)
    sc.build()
    rest = torch.from_numpy(np.concatenate([np.pad(m.xyz, ((0, 0), (0, 1))) for m in meshes], 0)).cuda()
    mats = torch.tensor([[0.6, -0.8, 0.0, 0.1, 0.8, 0.6, 0.0, -0.2, 0.0, 0.0, 1.0, 0.3]] * 3, dtype=torch.float32).cuda()
    sc.transform(rest.data_ptr(), mats.data_ptr())
    want = None
    for gl in (9, 10, 11):
        sc.set_tuning(refit_group_log2=gl)
        assert sc.tuning()["refit_group_log2"] == gl
        sc.refit()
        got = [t.aabb_tree().view(np.uint32).copy() for t in trees]
        if want is None:
            pos = [W.rigid_apply(m.xyz, mats[0].cpu().numpy()) for m in meshes]
            want = [Port.oibvh_refit(x, t.sorted_faces()[0]).view(np.uint32) for x, t in zip(pos, trees)]
        for g, wv in zip(got, want):
            assert np.array_equal(g, wv), gl


def test_full_batched_workload_parity(gpu):
    """The 512-pair workload at full size (103 M triangles): one captured frame
    gives the pair set of the plain path run pair by pair, and every pair's
    pair set and the frame's candidate count match the oracle's."""
    import torch

    from oibvh_gb300 import DeviceType, OibvhTree, Scene
    from oibvh_gb300 import workloads as W

    w = W.batched(512)
    trees = [OibvhTree(m) for m in w.rest]
    sc = Scene()
    for t in trees:
        sc.addOibvhTree(t)
    sc.set_pairs(w.pairs)
    sc.build()
    rest = torch.from_numpy(w.packed_rest_xyzw()).cuda()
    mats = torch.from_numpy(w.matrices(7)).cuda()
    sc.capture_frame(4, 3, True, rest.data_ptr(), mats.data_ptr())
    sc.launch_frame()
    sc.finish_frame()
    frame = sc.int_tri_pairs()
    assert frame.shape[0] > 100000
    # the plain path, pair by pair, on the same transformed positions
    parts = []
    for a, b in w.pairs:
        ps = Scene()
        ps.addOibvhTree(trees[a])
        ps.addOibvhTree(trees[b])
        ps.detectCollision(DeviceType.GPU0, 4, 3)
        h = ps.int_tri_pairs()
        h[:, 0], h[:, 1] = a, b
        parts.append(h)
    plain = np.concatenate(parts, 0)
    plain = plain[np.lexsort((plain[:, 3], plain[:, 2], plain[:, 1], plain[:, 0]))]
    assert np.array_equal(frame, plain)
    # every one of the 512 pairs against the oracle (host threads), and the
    # frame's candidate count against the oracle's total
    from tests_support import oracle_pair_sets

    pos = w.positions(7)
    want = oracle_pair_sets([(pos[a], w.rest[a].tri, pos[b], w.rest[b].tri) for a, b in w.pairs])
    for p, (a, b) in enumerate(w.pairs):
        got = frame[(frame[:, 0] == a) & (frame[:, 1] == b)][:, 2:]
        assert np.array_equal(got, want[p][0]), p
    assert sc.candidate_count() == sum(c for _, c in want)


def _with_unused_vertices(m, rng):
    """The same mesh with vertices no face uses scattered through its vertex
    array (and the used ones in a shuffled order)."""
    from oibvh_gb300 import meshes as M

    nV = m.xyz.shape[0]
    total = nV + int(rng.integers(1, nV + 2))
    where = rng.choice(total, nV, replace=False)
    xyz = rng.uniform(-2.0, 2.0, size=(total, 3)).astype(np.float32)
    xyz[where] = m.xyz
    return M.Mesh(xyz, where[m.tri.astype(np.int64)].astype(np.uint32))


def test_scene_build_renumbers_meshes_with_unused_vertices(gpu):
    """A scene build renumbers every tree's vertices in one set of launches
    (used vertices in first-use order, unused ones after them). Meshes whose
    vertex arrays hold unused vertices, built twice by their scene, keep the
    caller's numbering: sorted faces, refits from caller-order positions and
    pair sets equal the oracle's."""
    from oibvh_gb300 import DeviceType, OibvhTree, Scene
    from oibvh_gb300 import meshes as M
    from tests_support import soup

    rng = np.random.Generator(np.random.PCG64(31))
    base = [M.noise_displace(M.icosphere(3), 0.05, seed=3), M.icosphere(2, 0.9, (0.4, 0.1, 0.0)),
            soup(rng, 300, 0.1), M.grid_sheet(12, 1.5, 0.2, 0.5, origin=(-0.7, -0.7, 0.0)), soup(rng, 1, 0.3)]
    meshes = [_with_unused_vertices(m, rng) for m in base]
    trees = [OibvhTree(m) for m in meshes]
    sc = Scene()
    for t in trees:
        sc.addOibvhTree(t)
    sc.build()
    sc.build()  # a second renumbering on top of the first
    for t, m in zip(trees, meshes):
        aabbs, st, perm = Port.oibvh_build(m.xyz, m.tri)
        f, p = t.sorted_faces()
        assert np.array_equal(p, perm) and np.array_equal(f, st)
        assert np.array_equal(t.aabb_tree().view(np.uint32), aabbs.view(np.uint32))
    sc.detectCollision(DeviceType.GPU0, 4, 1)
    port = Port()
    for m in meshes:
        port.add_mesh(m.xyz, m.tri)
    want, wc = port.detect()
    assert np.array_equal(sc.int_tri_pairs(), sort_pairs(want)) and sc.candidate_count() == wc
    moved = [(m.xyz + rng.normal(scale=2e-3, size=m.xyz.shape)).astype(np.float32) for m in meshes]
    for t, x in zip(trees, moved):
        t.set_positions(x)
    sc.refit()
    for k, (t, x) in enumerate(zip(trees, moved)):
        st, _ = t.sorted_faces()
        assert np.array_equal(t.aabb_tree().view(np.uint32), Port.oibvh_refit(x, st).view(np.uint32)), k
        port.set_positions(k, x)
    sc.detectCollision(DeviceType.GPU0, 4, 1)
    want, wc = port.detect()
    assert np.array_equal(sc.int_tri_pairs(), sort_pairs(want)) and sc.candidate_count() == wc


def test_scene_build_launches_do_not_grow_with_trees(gpu):
    """Every stage of a scene build, the vertex renumbering included, is one
    launch for all trees: 3 and 60 trees take the same number of launches
    (both sort tree ids in one 8-bit radix pass)."""
    from oibvh_gb300 import OibvhTree, Scene
    from oibvh_gb300 import _native as N
    from oibvh_gb300 import meshes as M

    def launches(n):
        trees = [OibvhTree(M.noise_displace(M.icosphere(2 + k % 3), 0.05, seed=k)) for k in range(n)]
        sc = Scene()
        for t in trees:
            sc.addOibvhTree(t)
        sc.build()  # first build: tables uploaded
        before = N.lib().oibvh_get_launch_count()
        sc.build()
        return N.lib().oibvh_get_launch_count() - before

    assert launches(3) == launches(60)
