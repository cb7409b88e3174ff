"""Seeded input builders shared by the GPU tests."""
import numpy as np

from oibvh_gb300 import meshes as M


def soup(rng, n_tri, scale=0.25):
    base = rng.uniform(0.0, 1.0, size=(n_tri, 1, 3))
    off = rng.uniform(-scale, scale, size=(n_tri, 3, 3))
    xyz = (base + off).reshape(-1, 3).astype(np.float32)
    return M.Mesh(xyz, np.arange(3 * n_tri, dtype=np.uint32).reshape(-1, 3))


def soup_pair(seed):
    rng = np.random.Generator(np.random.PCG64(1000 + seed))
    sizes = [1, 2, 3, 7, 31, 64, 65, 300, 1000, 2049, 4095, 5000]
    na, nb = sizes[seed % len(sizes)], sizes[(seed * 7 + 3) % len(sizes)]
    return [soup(rng, na, 0.3 / max(1.0, na ** 0.33)), soup(rng, nb, 0.3 / max(1.0, nb ** 0.33))]


def mixed_scene(seed):
    rng = np.random.Generator(np.random.PCG64(2000 + seed))
    meshes = []
    n = 4 + seed % 3
    for k in range(n):
        kind = (seed + k) % 3
        if kind == 0:
            m = M.noise_displace(M.icosphere(int(rng.integers(1, 5))), 0.08, seed=int(rng.integers(1 << 30)))
        elif kind == 1:
            m = M.grid_sheet(int(rng.integers(4, 40)), 2.0, 0.2, float(rng.uniform(0.3, 1.0)), origin=(-1, -1, 0))
        else:
            m = soup(rng, int(rng.integers(1, 3000)), 0.05)
            m = M.Mesh((m.xyz * 2 - 1).astype(np.float32), m.tri)
        m = M.rigid_transform(m, M.random_rotation(rng), rng.uniform(-0.5, 0.5, 3))
        meshes.append(m)
    if seed % 2 == 0:
        pairs = None
    else:
        allp = [(i, j) for i in range(n) for j in range(n) if i != j]
        pick = rng.choice(len(allp), size=min(5, len(allp)), replace=False)
        pairs = np.array([allp[i] for i in pick], dtype=np.uint32)
    return meshes, pairs


def near_degenerate_pair(seed, n_tri=2000):
    """Triangles built to sit on the float/FP64 boundary: B holds, for each
    A triangle, one that shares an edge (folded by a tiny angle), one that is
    coplanar and shifted in-plane, one that touches at a vertex, and one lifted
    off the plane by a few ulps."""
    rng = np.random.Generator(np.random.PCG64(5000 + seed))
    base = rng.uniform(-1.0, 1.0, size=(n_tri, 1, 3))
    A = (base + rng.uniform(-0.05, 0.05, size=(n_tri, 3, 3))).astype(np.float64)
    out = []
    for t in A:
        p0, p1, p2 = t
        n = np.cross(p1 - p0, p2 - p0)
        n /= np.linalg.norm(n)
        eps = float(rng.choice([0.0, 1e-9, 1e-8, 1e-7, 1e-6]))
        # folded about edge p0-p1
        out.append([p0, p1, p2 + eps * n + (p0 - p2) * 0.5])
        # coplanar, shifted in-plane
        d = (p1 - p0) * rng.uniform(-0.6, 0.6)
        out.append([p0 + d, p1 + d, p2 + d])
        # touching at a vertex
        out.append([p2, p2 + (p2 - p0) * 0.7 + eps * n, p2 + (p2 - p1) * 0.7])
        # lifted by eps
        out.append([p0 + eps * n, p1 + eps * n, p2 + eps * n])
    B = np.asarray(out, dtype=np.float64)
    ma = M.Mesh(A.reshape(-1, 3).astype(np.float32), np.arange(3 * n_tri, dtype=np.uint32).reshape(-1, 3))
    mb = M.Mesh(B.reshape(-1, 3).astype(np.float32), np.arange(3 * len(out), dtype=np.uint32).reshape(-1, 3))
    return ma, mb


def morton63_order(xyz, tri):
    """Face order of a 63-bit-key build, restated in numpy: per face the
    centroid of its box, normalised by the mesh box (float32 operations in
    the build's order), 2^21 cells per axis, keys interleaved x << 2 | y << 1
    | z, then a stable sort by (key, face index)."""
    x = np.asarray(xyz, dtype=np.float32)
    t = np.asarray(tri, dtype=np.int64)
    bmin, bmax = x.min(0), x.max(0)
    v = x[t]                                      # [T, 3 vertices, 3 axes]
    mn, mx = v.min(1), v.max(1)
    centroid = (mn + mx) * np.float32(0.5)
    u = (centroid - bmin) / (bmax - bmin)
    q = np.clip(u * np.float32(2097152.0), np.float32(0.0), np.float32(2097151.0)).astype(np.uint64)

    def stretch(a):
        a = a & np.uint64(0x1FFFFF)
        a = (a | (a << np.uint64(32))) & np.uint64(0x1F00000000FFFF)
        a = (a | (a << np.uint64(16))) & np.uint64(0x1F0000FF0000FF)
        a = (a | (a << np.uint64(8))) & np.uint64(0x100F00F00F00F00F)
        a = (a | (a << np.uint64(4))) & np.uint64(0x10C30C30C30C30C3)
        a = (a | (a << np.uint64(2))) & np.uint64(0x1249249249249249)
        return a

    key = (stretch(q[:, 0]) << np.uint64(2)) | (stretch(q[:, 1]) << np.uint64(1)) | stretch(q[:, 2])
    return np.argsort(key, kind="stable").astype(np.uint32)


def bvtt_front_widths(ma, mb, start, steps=40):
    """Widths of the BVTT front, level by level, of the one-level-per-step
    traversal from the cross product of both trees' nodes at `start`: the
    number of overlapping node pairs that are not leaf x leaf after each
    expansion (a leaf stays put while the other side descends). Computed on
    the oracle's restatement of the GPU tree, so a test can show that a
    tuning reaches a given front shape."""
    from oracle.oracle import Port

    def shape(nT):
        p = 1 << max(0, (nT - 1).bit_length())
        return p.bit_length() - 1, p - nT

    def virtual_above(L, vl, l):
        if l == 0:
            return 0
        vc = vl >> (L - (l - 1))
        return (vc << 1) - bin(vc).count("1")

    trees = []
    for m in (ma, mb):
        boxes, _, _ = Port.oibvh_build(m.xyz, m.tri)
        L, vl = shape(m.tri.shape[0])
        va = np.array([virtual_above(L, vl, l) for l in range(L + 1)], dtype=np.int64)
        trees.append((boxes, L, vl, va))

    def level(i):
        return np.floor(np.log2(i + 1)).astype(np.int64)

    def box(t, i):
        boxes, L, vl, va = t
        return boxes[i - va[level(i)]]

    def keep(ia, ib):
        a, b = box(trees[0], ia), box(trees[1], ib)
        ov = np.all(a[:, :3] <= b[:, 3:], 1) & np.all(a[:, 3:] >= b[:, :3], 1)
        leaves = (level(ia) == trees[0][1]) & (level(ib) == trees[1][1])
        m = ov & ~leaves
        return ia[m], ib[m]

    def children(t, i):
        _, L, vl, _ = t
        li = level(i)
        leaf = li == L
        first = np.where(leaf, i, 2 * i + 1)
        nl = np.minimum(li + 1, L)
        right = (np.int64(2) << nl) - 2 - (vl >> (L - nl))
        return first, np.where(leaf, 1, np.minimum(2, right - first + 1))

    ea, eb = min(start, trees[0][1]), min(start, trees[1][1])
    na = (1 << ea) - (trees[0][2] >> (trees[0][1] - ea))
    nb = (1 << eb) - (trees[1][2] >> (trees[1][1] - eb))
    ia = np.repeat((1 << ea) - 1 + np.arange(na, dtype=np.int64), nb)
    ib = np.tile((1 << eb) - 1 + np.arange(nb, dtype=np.int64), na)
    ia, ib = keep(ia, ib)
    out = [int(ia.shape[0])]
    for _ in range(steps):
        if ia.shape[0] == 0:
            break
        fa, ca = children(trees[0], ia)
        fb, cb = children(trees[1], ib)
        xa, xb = [], []
        for x in (0, 1):
            for y in (0, 1):
                m = (x < ca) & (y < cb)
                xa.append((fa + x)[m])
                xb.append((fb + y)[m])
        ia, ib = keep(np.concatenate(xa), np.concatenate(xb))
        out.append(int(ia.shape[0]))
    return out


def oracle_pair_sets(jobs, threads=None):
    """The oracle's sorted (triA, triB) pair set and candidate count for each
    job (xyz_a, tri_a, xyz_b, tri_b), on host threads (the oracle's calls
    release the interpreter lock)."""
    import os
    import threading

    from oracle.oracle import Port, sort_pairs

    threads = threads or min(16, os.cpu_count() or 1)
    out = [None] * len(jobs)

    def work(k):
        for i in range(k, len(jobs), threads):
            xa, ta, xb, tb = jobs[i]
            p = Port()
            p.add_mesh(xa, ta)
            p.add_mesh(xb, tb)
            h, c = p.detect()
            out[i] = (sort_pairs(h)[:, 2:].copy(), c)

    ts = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return out
