"""Behaviour of the C ABI on the GPU: errors, split stages, copies, device
pointers, queue regrowth."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden
from oracle.oracle import Port, sort_pairs

pytestmark = pytest.mark.gpu


def _scene(meshes):
    from oibvh_gb300 import OibvhTree, Scene

    trees = [OibvhTree(m) for m in meshes]
    for t in trees:
        t.build()
    sc = Scene()
    for t in trees:
        sc.addOibvhTree(t)
    return sc, trees


def test_cpu_device_type_is_refused(gpu):
    from oibvh_gb300 import DeviceType, OibvhError

    g = load_golden("config1")
    sc, _ = _scene(g["meshes"])
    with pytest.raises(OibvhError) as e:
        sc.detectCollision(DeviceType.CPU, 4, 3)
    assert e.value.status == 6


def test_bad_arguments(gpu):
    from oibvh_gb300 import DeviceType, OibvhError, OibvhTree, Scene

    g = load_golden("config1")
    sc, trees = _scene(g["meshes"])
    with pytest.raises(OibvhError) as e:
        sc.detectCollision(DeviceType.GPU0, 4, 0)
    assert e.value.status == 1
    with pytest.raises(OibvhError):
        sc.set_pairs([(0, 0)])
    with pytest.raises(OibvhError):
        sc.set_pairs([(0, 5)])
    unbuilt = OibvhTree(g["meshes"][0])
    other = Scene()
    other.addOibvhTree(unbuilt)  # allowed: oibvh_scene_build builds scene trees together
    other.addOibvhTree(trees[0])
    with pytest.raises(OibvhError) as e:
        other.detectCollision(DeviceType.GPU0, 0, 1)
    assert e.value.status == 5
    with pytest.raises(OibvhError):
        unbuilt.refit()


def test_broad_then_narrow_equals_detect(gpu):
    from oibvh_gb300 import DeviceType

    g = load_golden("config1")
    sc, trees = _scene(g["meshes"])
    sc.broad(DeviceType.GPU0, 4, 3)
    assert sc.candidate_count() == g["candidates"][0]
    cands = sc.candidates()
    assert cands.shape == (g["candidates"][0], 4)
    # candidates are leaf pairs in Morton order: map to original faces and
    # check against the oracle's leaf-box overlap set
    perms = [t.sorted_faces()[1] for t in trees]
    orig = np.stack([perms[0][cands[:, 2]], perms[1][cands[:, 3]]], 1)
    assert len({tuple(r) for r in orig}) == orig.shape[0]
    sc.narrow()
    assert np.array_equal(sc.int_tri_pairs(), g["hits"][0])


def test_queue_regrowth(gpu):
    from oibvh_gb300 import DeviceType

    g = load_golden("identical")
    sc, _ = _scene(g["meshes"])
    sc.set_queue_capacity(front=8, candidates=8, hits=4)
    sc.detectCollision(DeviceType.GPU0, 2, 1)
    assert np.array_equal(sc.int_tri_pairs(), g["hits"][0])
    assert sc.stats()["retries"] >= 1


def test_copy_tree_then_refit(gpu):
    """OibvhTree(other, mesh) + refit, the sequence of src/main.cpp:129-135."""
    from oibvh_gb300 import DeviceType, OibvhTree, Scene
    from oibvh_gb300 import meshes as M

    a = M.noise_displace(M.icosphere(4), 0.05, seed=3)
    b = M.Mesh(a.xyz + np.array([1.0, 0.0, 0.0], np.float32), a.tri)  # translate(+1, 0, 0)
    ta = OibvhTree(a)
    ta.build()
    tb = OibvhTree.copy_of(ta, b)
    tb.refit()
    sc = Scene()
    sc.addOibvhTree(ta)
    sc.addOibvhTree(tb)
    sc.detectCollision(DeviceType.GPU0, 4, 3)
    p = Port()
    p.add_mesh(a.xyz, a.tri)
    p.add_mesh(b.xyz, b.tri)
    want, wc = p.detect()
    assert np.array_equal(sc.int_tri_pairs(), sort_pairs(want))
    assert sc.candidate_count() == wc
    assert sc.getIntTriPairCount() == want.shape[0]


def test_refit_from_device_pointer(gpu):
    import torch

    from oibvh_gb300 import DeviceType

    g = load_golden("deforming")
    sc, trees = _scene(g["meshes"])
    fr = g["frames"][1]
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in fr]
    torch.cuda.synchronize()
    for t, d in zip(trees, dev):
        t.refit_device(d.data_ptr())
    sc.detectCollision(DeviceType.GPU0, 4, 3)
    assert np.array_equal(sc.int_tri_pairs(), g["hits"][2])


def test_one_triangle_meshes(gpu):
    from oibvh_gb300 import DeviceType
    from oibvh_gb300 import meshes as M

    a = M.Mesh(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([[0, 1, 2]], np.uint32))
    b = M.Mesh(np.array([[0.2, 0.2, -1], [0.2, 0.2, 1], [0.3, 0.1, 0]], np.float32), np.array([[0, 1, 2]], np.uint32))
    sc, trees = _scene([a, b])
    assert trees[0].size == 1 and trees[0].getDepth() == 0
    sc.detectCollision(DeviceType.GPU0, 0, 1)
    assert sc.int_tri_pairs().tolist() == [[0, 1, 0, 0]]


def test_stream_argument(gpu):
    import torch

    from oibvh_gb300 import DeviceType

    g = load_golden("noise_spheres")
    sc, trees = _scene(g["meshes"])
    s = torch.cuda.Stream()
    sc.detectCollision(DeviceType.GPU0, 4, 3, stream=s)
    assert np.array_equal(sc.int_tri_pairs(), g["hits"][0])


def test_positions_xyzw_by_reference(gpu):
    """oibvh_tree_set_positions4_device: 16-byte (x, y, z, w) records in the
    caller's vertex order, kept by reference and read again by every refit
    (the tree's own vertex numbering differs after the build)."""
    import torch

    from oibvh_gb300 import DeviceType

    g = load_golden("deforming")
    sc, trees = _scene(g["meshes"])
    fr = g["frames"][0]
    dev = [torch.nn.functional.pad(torch.from_numpy(np.ascontiguousarray(x)), (0, 1)).contiguous().cuda() for x in fr]
    for t, d in zip(trees, dev):
        t.set_positions4_device(d.data_ptr())
    sc.refit()
    sc.detectCollision(DeviceType.GPU0, 4, 3)
    assert np.array_equal(sc.int_tri_pairs(), g["hits"][1])
    # the same buffers, new contents: the next refit reads them
    for d, x in zip(dev, g["frames"][1]):
        d[:, :3].copy_(torch.from_numpy(np.ascontiguousarray(x)).cuda())
    torch.cuda.synchronize()
    sc.refit()
    sc.detectCollision(DeviceType.GPU0, 4, 3)
    assert np.array_equal(sc.int_tri_pairs(), g["hits"][2])
    # misaligned pointer is refused
    from oibvh_gb300 import OibvhError

    with pytest.raises(OibvhError):
        trees[0].set_positions4_device(dev[0].data_ptr() + 4)


def test_obj_meshes_through_the_pipeline(gpu, tmp_path):
    """A mesh read from an OBJ file collides exactly as the oracle says."""
    import numpy as np

    from oibvh_gb300 import DeviceType, OibvhTree, Scene
    from oibvh_gb300 import meshes as M
    from oracle.oracle import Port, sort_pairs

    a = M.noise_displace(M.icosphere(4), 0.05, seed=1)
    b = M.rigid_transform(M.noise_displace(M.icosphere(4), 0.05, seed=2), np.eye(3), (0.9, 0.1, 0.0))
    paths = [str(tmp_path / "a.obj"), str(tmp_path / "b.obj")]
    for m, p in zip((a, b), paths):
        M.save_obj(m, p)
    meshes = [M.load_obj(p) for p in paths]
    trees = [OibvhTree(m) for m in meshes]
    sc = Scene()
    for t in trees:
        t.build()
        sc.addOibvhTree(t)
    sc.detectCollision(DeviceType.GPU0, 4, 3)
    port = Port()
    for m in meshes:
        port.add_mesh(m.xyz, m.tri)
    want, _ = port.detect()
    assert np.array_equal(sc.int_tri_pairs(), sort_pairs(want))
    assert want.shape[0] > 0


def test_empty_and_single_tree_scenes(gpu):
    """A scene with no trees, or one tree (no pair), detects nothing, and an
    explicit empty pair list detects nothing either."""
    import numpy as np

    from oibvh_gb300 import DeviceType, OibvhTree, Scene
    from oibvh_gb300 import meshes as M

    sc = Scene()
    sc.detectCollision(DeviceType.GPU0, 0, 1)
    assert sc.getIntTriPairCount() == 0
    t = OibvhTree(M.icosphere(2))
    t.build()
    sc.addOibvhTree(t)
    sc.detectCollision(DeviceType.GPU0, 4, 3)
    assert sc.getIntTriPairCount() == 0 and sc.int_tri_pairs().shape == (0, 4)
    u = OibvhTree(M.icosphere(2, 1.0, (0.5, 0.0, 0.0)))
    u.build()
    sc.addOibvhTree(u)
    sc.set_pairs(np.zeros((0, 2), dtype=np.uint32))
    sc.detectCollision(DeviceType.GPU0, 0, 1)
    assert sc.getIntTriPairCount() == 0


def test_maximum_tree_size(gpu):
    """2^23 triangles, the largest mesh a tree takes (24-bit node indices in
    the BVTT records), against a small sphere crossing it: the oracle's pair
    set; one more triangle is refused."""
    import numpy as np

    from oibvh_gb300 import DeviceType, OibvhError, OibvhTree, Scene
    from oibvh_gb300 import meshes as M
    from oracle.oracle import Port, sort_pairs

    sheet = M.grid_sheet(2048, 2.0, 0.0, 1.0, origin=(-1.0, -1.0, 0.0))
    assert sheet.n_triangles == 1 << 23
    ball = M.icosphere(3, 0.3, (0.1, -0.2, 0.05))
    trees = [OibvhTree(sheet), OibvhTree(ball)]
    sc = Scene()
    for t in trees:
        t.build()
        sc.addOibvhTree(t)
    assert trees[0].getPrimCount() == 1 << 23
    sc.detectCollision(DeviceType.GPU0, 4, 3)
    port = Port()
    port.add_mesh(sheet.xyz, sheet.tri)
    port.add_mesh(ball.xyz, ball.tri)
    want, wc = port.detect()
    assert want.shape[0] > 0
    assert np.array_equal(sc.int_tri_pairs(), sort_pairs(want))
    assert sc.candidate_count() == wc
    big = M.Mesh(np.zeros((3, 3), np.float32), np.zeros(((1 << 23) + 1, 3), np.uint32))
    with pytest.raises(OibvhError):
        OibvhTree(big)


def test_rebuild_and_scene_build_keep_caller_numbering(gpu):
    """A tree built twice, then built again by its scene (each build renumbers
    the vertices on top of the last): sorted faces still come back in the
    caller's vertex numbering, and positions set afterwards in the caller's
    order give the oracle's pair sets."""
    from oibvh_gb300 import DeviceType, OibvhTree, Scene

    g = load_golden("deforming")
    trees = [OibvhTree(m) for m in g["meshes"]]
    for t in trees:
        t.build()
        t.build()
    for t, m in zip(trees, g["meshes"]):
        _, st, perm = Port.oibvh_build(m.xyz, m.tri)
        f, p = t.sorted_faces()
        assert np.array_equal(f, st) and np.array_equal(p, perm)
    sc = Scene()
    for t in trees:
        sc.addOibvhTree(t)
    sc.build()
    for t, m in zip(trees, g["meshes"]):
        _, st, _ = Port.oibvh_build(m.xyz, m.tri)
        assert np.array_equal(t.sorted_faces()[0], st)
    sc.detectCollision(DeviceType.GPU0, 4, 3)
    assert np.array_equal(sc.int_tri_pairs(), g["hits"][0])
    for f, fr in enumerate(g["frames"]):
        for t, x in zip(trees, fr):
            t.refit(x)
        sc.detectCollision(DeviceType.GPU0, 4, 3)
        assert np.array_equal(sc.int_tri_pairs(), g["hits"][f + 1]), f
