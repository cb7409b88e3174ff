"""oibvh_pair_detect_noalloc, the allocation-free detect, against oibvh_scene_detect.

The allocation-free entry point is for callers that may not allocate while they
run: a frame loop with a hard time budget (cudaMalloc may synchronise the whole
device and take an unbounded time), or an application whose device memory is
all reserved by an outside pool allocator. It walks the same kernels over a
fixed scratch area compiled into the library, so its pair set must equal the
growing-queue detect's bit for bit. Two calls in a row (with a refit in between) also show
that the shared scratch left by one call does not leak into the next.

This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _sorted(rec):
    rec = np.asarray(rec, dtype=np.uint32).reshape(-1, 4)
    return rec[np.lexsort((rec[:, 3], rec[:, 2], rec[:, 1], rec[:, 0]))] if rec.shape[0] else rec


def test_noalloc_detect_equals_scene_detect_two_calls(gpu):
    import torch

    from oibvh_gb300 import DeviceType, OibvhTree, Scene
    from oibvh_gb300 import _native as N

    g = load_golden("deforming")
    trees = [OibvhTree(m) for m in g["meshes"]]
    for t in trees:
        t.build()
    scene = Scene()
    for t in trees:
        scene.addOibvhTree(t)

    cap = 1 << 16
    out = torch.empty((cap, 4), dtype=torch.int32, device="cuda")  # the caller owns the output buffer
    frames = [None, g["frames"][0]]  # rest positions, then one refit frame
    for call, frame in enumerate(frames):
        if frame is not None:
            for t, xyz in zip(trees, frame):
                t.refit(xyz)
        scene.detectCollision(DeviceType.GPU0, 4, 3)
        want = scene.int_tri_pairs()
        assert want.shape[0] > 0

        out.fill_(-1)
        torch.cuda.synchronize()
        n = ctypes.c_uint32(0)
        st = N.lib().oibvh_pair_detect_noalloc(trees[0].handle, trees[1].handle, 4,
                                               ctypes.c_void_p(out.data_ptr()), cap, ctypes.byref(n), None)
        assert st == 0, N.lib().oibvh_last_error().decode()
        got = _sorted(out[: n.value].cpu().numpy().view(np.uint32))
        assert np.array_equal(got, want), f"call {call}: {got.shape[0]} pairs, expected {want.shape[0]}"
        assert np.array_equal(got, g["hits"][call])  # and the reference's pair set


def test_noalloc_detect_reports_a_short_output_buffer(gpu):
    import torch

    from oibvh_gb300 import OibvhTree
    from oibvh_gb300 import _native as N

    g = load_golden("config1")
    trees = [OibvhTree(m) for m in g["meshes"]]
    for t in trees:
        t.build()
    out = torch.empty((8, 4), dtype=torch.int32, device="cuda")
    n = ctypes.c_uint32(0)
    st = N.lib().oibvh_pair_detect_noalloc(trees[0].handle, trees[1].handle, 0, ctypes.c_void_p(out.data_ptr()), 8,
                                           ctypes.byref(n), None)
    assert st == N.ERR_OVERFLOW
    assert n.value == g["hits"][0].shape[0]
