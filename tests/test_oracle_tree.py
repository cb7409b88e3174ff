"""The oibvh tree restatement (reference GPU build layout) is self-consistent."""
import numpy as np
import pytest

from oracle.oracle import Port


def next_pow2(x):
    p = 1
    while p < x:
        p *= 2
    return p


def level_counts(T):
    L = next_pow2(T).bit_length() - 1
    vl = next_pow2(T) - T
    return L, [(1 << l) - (vl >> (L - l)) for l in range(L + 1)]


@pytest.mark.parametrize("T", list(range(1, 70)) + [127, 128, 129, 1000, 4097])
def test_tree_levels(T):
    rng = np.random.default_rng(T)
    V = T + 3
    xyz = rng.normal(size=(V, 3)).astype(np.float32)
    tri = rng.integers(0, V, size=(T, 3)).astype(np.uint32)
    aabbs, st, perm = Port.oibvh_build(xyz, tri)
    L, cnt = level_counts(T)
    # oibvh_get_size (include/cuda/oibvh.cuh:56-59): 2T + popcount(nextpow2(T)-T) - 1
    expect_size = 1 if T == 1 else 2 * T + bin(next_pow2(T) - T).count("1") - 1
    assert aabbs.shape[0] == sum(cnt) == expect_size
    # stable Morton order
    codes = Port.morton_codes(xyz, tri)
    assert np.array_equal(perm, np.argsort(codes, kind="stable"))
    assert np.array_equal(st, tri[perm])
    # every internal node is the exact union of its real children
    off = np.concatenate([[0], np.cumsum(cnt)])
    for l in range(L):
        for j in range(cnt[l]):
            ch = [2 * j] + ([2 * j + 1] if 2 * j + 1 < cnt[l + 1] else [])
            kids = aabbs[off[l + 1] + np.array(ch)]
            node = aabbs[off[l] + j]
            assert np.array_equal(node[:3], kids[:, :3].min(0)) and np.array_equal(node[3:], kids[:, 3:].max(0))
    # leaves are the sorted faces' boxes
    leaf = aabbs[off[L]:]
    v = xyz[st]
    assert np.array_equal(leaf[:, :3], v.min(1)) and np.array_equal(leaf[:, 3:], v.max(1))


def test_morton_matches_numpy():
    from oibvh_gb300 import meshes as M

    m = M.noise_displace(M.icosphere(3), 0.05, seed=1)
    codes = Port.morton_codes(m.xyz, m.tri)
    v = m.xyz[m.tri]
    mn, mx = v.min(1), v.max(1)
    bmin, bmax = m.xyz.min(0), m.xyz.max(0)
    c = (mn + mx) * np.float32(0.5)
    u = (c - bmin) / (bmax - bmin)
    q = np.clip(u * np.float32(1024.0), 0, 1023).astype(np.uint32)

    def stretch(x):
        x = x & 0x3FF
        x = (x | (x << 16)) & 0x30000FF
        x = (x | (x << 8)) & 0x300F00F
        x = (x | (x << 4)) & 0x30C30C3
        x = (x | (x << 2)) & 0x9249249
        return x

    want = (stretch(q[:, 0]) << 2) | (stretch(q[:, 1]) << 1) | stretch(q[:, 2])
    assert np.array_equal(codes, want.astype(np.uint32))
