"""Out-of-memory paths, driven on a healthy GPU through the library's test
hook oibvh_debug_fail_alloc_after(n): the n-th allocation the library attempts
from then on fails as cudaMalloc would (cudaErrorMemoryAllocation) without
calling CUDA. Every allocation of tree creation and build, scene detect
(including queue regrowth), frame capture and the server (creation, the
lane buffers allocated at start, a batch's reallocated queues) is made to
fail in turn: the call reports
OIBVH_ERR_OOM, and afterwards the same handles work and give the oracle's
pair sets (or are destroyed cleanly). The reference ignores every CUDA error
(include/cuda/utils.cuh:6-34) and has no such path."""
import numpy as np
import pytest

from conftest import load_golden
from oracle.oracle import Port, sort_pairs

pytestmark = pytest.mark.gpu


def _N():
    from oibvh_gb300 import _native as N

    return N


@pytest.fixture(autouse=True)
def _hook_off(gpu):
    _N().lib().oibvh_debug_fail_alloc_after(-1)
    yield
    _N().lib().oibvh_debug_fail_alloc_after(-1)


def _attempts(fn):
    """Allocations `fn` attempts (the hook off)."""
    L = _N().lib()
    a0 = L.oibvh_debug_alloc_attempts()
    fn()
    return int(L.oibvh_debug_alloc_attempts() - a0)


def _expect_oom(n, fn):
    N = _N()
    N.lib().oibvh_debug_fail_alloc_after(n)
    with pytest.raises(N.OibvhError) as e:
        fn()
    N.lib().oibvh_debug_fail_alloc_after(-1)
    assert e.value.status == N.ERR_OOM, f"allocation {n}: {e.value}"


def test_tree_create_and_build_report_oom_then_work():
    from oibvh_gb300 import DeviceType, OibvhTree, Scene

    g = load_golden("deforming")
    ma, mb = g["meshes"]
    k = _attempts(lambda: OibvhTree(ma))
    assert k >= 5
    for n in range(k):
        _expect_oom(n, lambda: OibvhTree(ma))
    t = OibvhTree(ma)
    kb = _attempts(lambda: OibvhTree(ma).build())
    kb -= k  # the creation's share
    assert kb >= 1
    for n in range(kb):
        _expect_oom(n, t.build)
    t.build()
    aabbs, st, perm = Port.oibvh_build(ma.xyz, ma.tri)
    f, p = t.sorted_faces()
    assert np.array_equal(p, perm) and np.array_equal(f, st)
    assert np.array_equal(t.aabb_tree().view(np.uint32), aabbs.view(np.uint32))
    tb = OibvhTree(mb)
    tb.build()
    sc = Scene()
    sc.addOibvhTree(t)
    sc.addOibvhTree(tb)
    sc.detectCollision(DeviceType.GPU0, 4, 3)
    assert np.array_equal(sc.int_tri_pairs(), g["hits"][0])


def _scene(g):
    from oibvh_gb300 import OibvhTree, Scene

    trees = [OibvhTree(m) for m in g["meshes"]]
    for t in trees:
        t.build()
    sc = Scene()
    for t in trees:
        sc.addOibvhTree(t)
    return sc, trees


def test_scene_detect_and_queue_regrowth_report_oom_then_work():
    from oibvh_gb300 import DeviceType

    g = load_golden("deforming")

    def fresh(small):
        sc, trees = _scene(g)
        if small:
            sc.set_queue_capacity(front=16, hits=8)  # the first detect regrows both
        return sc, trees

    for small in (False, True):
        sc0, _ = fresh(small)
        k = _attempts(lambda: sc0.detectCollision(DeviceType.GPU0, 4, 3))
        assert k >= 3
        for n in range(k):
            sc, trees = fresh(small)
            _expect_oom(n, lambda: sc.detectCollision(DeviceType.GPU0, 4, 3))
            sc.detectCollision(DeviceType.GPU0, 4, 3)  # the same scene, the hook off
            assert np.array_equal(sc.int_tri_pairs(), g["hits"][0]), (small, n)
            assert sc.candidate_count() == g["candidates"][0]


def test_frame_capture_reports_oom_then_works():
    import torch

    from oibvh_gb300 import OibvhTree, Scene
    from oibvh_gb300 import workloads as W

    w = W.batched(6, seed=21, subdivs=(2, 3), variants=2)
    rest = torch.from_numpy(w.packed_rest_xyzw()).cuda()
    mats = torch.from_numpy(w.matrices(3)).cuda()
    port = Port()
    for x, m in zip(w.positions(3), w.rest):
        port.add_mesh(x, m.tri)
    want, wc = port.detect(np.asarray(w.pairs, dtype=np.uint32))
    want = sort_pairs(want)

    def fresh():
        trees = [OibvhTree(m) for m in w.rest]
        sc = Scene()
        for t in trees:
            sc.addOibvhTree(t)
        sc.set_pairs(w.pairs)
        sc.build()
        return sc, trees

    sc0, _ = fresh()
    k = _attempts(lambda: sc0.capture_frame(0, 1, True, rest.data_ptr(), mats.data_ptr()))
    assert k >= 3
    for n in range(k):
        sc, trees = fresh()
        _expect_oom(n, lambda: sc.capture_frame(0, 1, True, rest.data_ptr(), mats.data_ptr()))
        sc.capture_frame(0, 1, True, rest.data_ptr(), mats.data_ptr())
        sc.launch_frame()
        sc.finish_frame()
        assert np.array_equal(sc.int_tri_pairs(), want), n
        assert sc.candidate_count() == wc


def test_server_creation_and_batch_report_oom_then_serve():
    from oibvh_gb300 import OibvhTree, Server
    from oibvh_gb300 import meshes as M
    from oibvh_gb300 import workloads as W

    N = _N()
    meshes = [W.noise_displace_mesh(3, 0.05, 31), W.noise_displace_mesh(2, 0.05, 32)]
    trees = [OibvhTree(m) for m in meshes]
    for t in trees:
        t.build()
    k = _attempts(lambda: Server(0, 64 << 20, 16, 2).close())
    assert k >= 1
    for n in range(k):
        _expect_oom(n, lambda: Server(0, 64 << 20, 16, 2))
    mat = np.concatenate([M.random_rotation(np.random.default_rng(4)), [[0.3], [0.1], [0.0]]], 1).astype(np.float32)
    p = Port()
    p.add_mesh(meshes[0].xyz, meshes[0].tri)
    p.add_mesh(W.rigid_apply(meshes[1].xyz, mat.reshape(12)), meshes[1].tri)
    h, _ = p.detect()
    want = sort_pairs(h)[:, 2:]
    assert want.shape[0] > 0
    def pool_server():
        srv = Server(0, 64 << 20, 16, 1)
        for t in trees:
            srv.add_mesh(t)
        return srv

    # start allocates every lane's buffers: each of its allocations fails in
    # turn, and a later start on the same server succeeds
    srv = pool_server()
    ks = _attempts(srv.start)
    srv.close()
    assert ks >= 10
    for n in range(0, ks, 3):
        srv = pool_server()
        _expect_oom(n, srv.start)
        srv.start()
        t1 = srv.submit(0, 1, mat)
        srv.wait(t1)
        assert np.array_equal(srv.pairs(t1), want)
        srv.release(t1)
        srv.close()
    # new queue capacities: the next batch reallocates its lane's queues, and
    # that allocation fails
    srv = pool_server()
    srv.start()
    srv.set_queue_capacity(64, 64)
    N.lib().oibvh_debug_fail_alloc_after(0)
    t0 = srv.submit(0, 1, mat)
    with pytest.raises(N.OibvhError) as e:
        srv.wait(t0)
    assert e.value.status == N.ERR_OOM
    N.lib().oibvh_debug_fail_alloc_after(-1)
    srv.release(t0)
    for _ in range(2):  # the lane starts clean: later queries are served (queues regrown)
        t1 = srv.submit(0, 1, mat)
        srv.wait(t1)
        assert np.array_equal(srv.pairs(t1), want)
        srv.release(t1)
    assert srv.stats()["redos"] >= 1
    srv.close()
