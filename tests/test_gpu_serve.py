"""The serving loop (oibvh_server_*): continuous batching over a pool of
resident meshes. Every query's pair set must be the oracle's for that pair
(B under its rigid transform against A at rest), the same when the query
runs alone and when it runs in a mix with others, and admission must respect
the memory budget."""
import threading

import numpy as np
import pytest

from oracle.oracle import Port, sort_pairs

pytestmark = pytest.mark.gpu


def _pool(n=12, seed=3):
    from oibvh_gb300 import workloads as W

    rng = np.random.Generator(np.random.PCG64(seed))
    meshes = []
    for k in range(n):
        s = int(rng.integers(1, 5))
        m = W.noise_displace_mesh(s, 0.05, seed * 100 + k)
        meshes.append(m)
    return meshes


def _queries(n_mesh, n_q, seed=9):
    from oibvh_gb300 import meshes as M

    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n_q):
        a, b = (int(x) for x in rng.integers(0, n_mesh, 2))
        R = M.random_rotation(rng)
        t = rng.uniform(-1.2, 1.2, 3)
        out.append((a, b, np.concatenate([R, t[:, None]], 1).astype(np.float32).reshape(12)))
    return out


def _oracle(meshes, q):
    from oibvh_gb300 import workloads as W

    a, b, mat = q
    p = Port()
    p.add_mesh(meshes[a].xyz, meshes[a].tri)
    p.add_mesh(W.rigid_apply(meshes[b].xyz, mat), meshes[b].tri)
    h, _ = p.detect()
    h = sort_pairs(h)
    return h[:, 2:].copy()


def _server(meshes, budget=256 << 20, max_batch=64, lanes=3):
    from oibvh_gb300 import OibvhTree, Server

    trees = [OibvhTree(m) for m in meshes]
    for t in trees:
        t.build()
    srv = Server(0, budget, max_batch, lanes)
    for t in trees:
        srv.add_mesh(t)
    srv.start()
    return srv


def _run_alone(srv, qs):
    out = []
    for a, b, m in qs:
        t = srv.submit(a, b, m)
        info = srv.wait(t)
        assert info["batch_size"] == 1
        out.append(srv.pairs(t))
        srv.release(t)
    return out


def _run_mix(srv, qs):
    tickets = [srv.submit(a, b, m) for a, b, m in qs]
    out, sizes = [], []
    for t in tickets:
        info = srv.wait(t)
        sizes.append(info["batch_size"])
        out.append(srv.pairs(t))
        srv.release(t)
    return out, sizes


def test_results_alone_and_in_the_mix_equal_the_oracle(gpu):
    meshes = _pool()
    qs = _queries(len(meshes), 48)
    srv = _server(meshes)
    alone = _run_alone(srv, qs)
    mix, sizes = _run_mix(srv, qs)
    assert max(sizes) > 1  # the mix did batch
    hits = 0
    for k, q in enumerate(qs):
        want = _oracle(meshes, q)
        assert np.array_equal(alone[k], want), f"query {k} alone"
        assert np.array_equal(mix[k], want), f"query {k} in the mix"
        hits += want.shape[0]
    assert hits > 0
    st = srv.stats()
    assert st["completed"] == 2 * len(qs) and st["failed"] == 0
    srv.close()


def test_admission_by_memory_budget(gpu):
    """A budget that holds only a few slots: every query still completes,
    the arena never exceeds the budget, and an oversized query is refused."""
    from oibvh_gb300 import OibvhError, OibvhTree, Server
    from oibvh_gb300 import workloads as W

    meshes = _pool(6, seed=5)
    big = W.noise_displace_mesh(6, 0.05, 77)  # 81,920 triangles: ~3.3 MB slot
    trees = [OibvhTree(m) for m in meshes + [big]]
    for t in trees:
        t.build()
    budget = 2 << 20
    srv = Server(0, budget, 64, 2)
    for t in trees:
        srv.add_mesh(t)
    srv.start()
    qs = _queries(len(meshes), 40, seed=21)
    mix, _ = _run_mix(srv, qs)
    for k, q in enumerate(qs):
        assert np.array_equal(mix[k], _oracle(meshes, q))
    st = srv.stats()
    assert st["arena_peak_bytes"] <= st["arena_bytes"] and st["arena_used_bytes"] == 0
    with pytest.raises(OibvhError):
        srv.submit(0, len(meshes), np.eye(3, 4, dtype=np.float32))
    srv.close()


def test_small_queues_are_regrown_not_truncated(gpu):
    meshes = _pool(6, seed=8)
    qs = _queries(len(meshes), 16, seed=4)
    srv = _server(meshes, lanes=2)
    srv.set_queue_capacity(front=64, hits=16)
    mix, _ = _run_mix(srv, qs)
    for k, q in enumerate(qs):
        assert np.array_equal(mix[k], _oracle(meshes, q))
    assert srv.stats()["redos"] > 0
    srv.close()


def test_concurrent_submitters(gpu):
    meshes = _pool(8, seed=12)
    qs = _queries(len(meshes), 64, seed=31)
    srv = _server(meshes, lanes=4)
    results = {}

    def client(lo, hi):
        tickets = [(k, srv.submit(*qs[k])) for k in range(lo, hi)]
        for k, t in tickets:
            srv.wait(t)
            results[k] = srv.pairs(t)
            srv.release(t)

    th = [threading.Thread(target=client, args=(16 * i, 16 * i + 16)) for i in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for k, q in enumerate(qs):
        assert np.array_equal(results[k], _oracle(meshes, q)), k
    srv.close()


def test_batch_cost_limit(gpu):
    """With a one-triangle batch budget every query runs alone, and results
    stay those of the oracle."""
    meshes = _pool(6, seed=14)
    qs = _queries(len(meshes), 20, seed=8)
    srv = _server(meshes, lanes=2)
    srv.set_batch_cost(1)
    mix, sizes = _run_mix(srv, qs)
    assert max(sizes) == 1
    for k, q in enumerate(qs):
        assert np.array_equal(mix[k], _oracle(meshes, q))
    srv.close()
