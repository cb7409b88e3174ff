"""The C-ABI library loads, exports every symbol the header declares, and
rejects bad arguments before touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "oibvh_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(oibvh_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_reference_surface():
    names = declared_functions()
    for must in ["oibvh_tree_create", "oibvh_tree_build", "oibvh_tree_refit", "oibvh_scene_add_tree",
                 "oibvh_scene_detect", "oibvh_scene_get_int_tri_pair_count", "oibvh_scene_get_int_tri_pairs"]:
        assert must in names


def test_library_exports_every_declared_symbol():
    from oibvh_gb300 import _native

    L = _native.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
    bound = {n for n, _, _ in _native.SIGNATURES}
    assert bound == set(declared_functions())
    assert L.oibvh_version() >= 100


def test_library_has_sm103a_code_only():
    from oibvh_gb300 import build

    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_argument_errors_need_no_gpu():
    from oibvh_gb300 import _native as N

    L = N.lib()
    h = ctypes.c_void_p()
    xyz = np.zeros((3, 3), np.float32)
    tri = np.array([[0, 1, 2]], np.uint32)
    bad = np.array([[0, 1, 3]], np.uint32)
    f32 = lambda a: a.ctypes.data_as(N._f32p)  # noqa: E731
    u32 = lambda a: a.ctypes.data_as(N._u32p)  # noqa: E731
    assert L.oibvh_tree_create(f32(xyz), 3, u32(tri), 0, 0, ctypes.byref(h)) == N.ERR_ARG
    assert L.oibvh_tree_create(f32(xyz), 3, u32(bad), 1, 0, ctypes.byref(h)) == N.ERR_ARG
    assert b"vertex 3" in L.oibvh_last_error()
    assert L.oibvh_tree_create(None, 3, u32(tri), 1, 0, ctypes.byref(h)) == N.ERR_ARG
    assert L.oibvh_tree_create(f32(xyz), 3, u32(tri), 1, 0, None) == N.ERR_ARG
    assert L.oibvh_scene_detect(None, 0, 0, 1, None) == N.ERR_ARG
    assert L.oibvh_status_string(N.ERR_OVERFLOW) == b"queue overflow"


def test_extension_argument_errors_need_no_gpu():
    """Serving, precision, tuning and Morton-width entry points reject bad
    arguments before any CUDA call."""
    from oibvh_gb300 import _native as N

    L = N.lib()
    h = ctypes.c_void_p()
    # server: null out, a budget under 1 MiB, no batch, no lane, too many lanes
    assert L.oibvh_server_create(0, 1 << 30, 64, 4, None) == N.ERR_ARG
    assert L.oibvh_server_create(0, 1 << 10, 64, 4, ctypes.byref(h)) == N.ERR_ARG
    assert L.oibvh_server_create(0, 1 << 30, 0, 4, ctypes.byref(h)) == N.ERR_ARG
    assert L.oibvh_server_create(0, 1 << 30, 64, 0, ctypes.byref(h)) == N.ERR_ARG
    assert L.oibvh_server_create(0, 1 << 30, 64, 17, ctypes.byref(h)) == N.ERR_ARG
    mat = np.eye(3, 4, dtype=np.float32)
    t = ctypes.c_uint64()
    assert L.oibvh_server_submit(None, 0, 1, mat.ctypes.data_as(N._f32p), ctypes.byref(t)) == N.ERR_ARG
    assert L.oibvh_server_wait(None, 1, 10, None) == N.ERR_ARG
    assert L.oibvh_server_release(None, 1) == N.ERR_ARG
    assert L.oibvh_server_start(None) == N.ERR_ARG
    assert L.oibvh_server_destroy(None) == N.OK
    # scene-level knobs on a null scene
    assert L.oibvh_scene_set_precision(None, 1) == N.ERR_ARG
    assert L.oibvh_scene_get_precision(None) == -1
    assert L.oibvh_scene_set_tuning(None, None) == N.ERR_ARG
    assert L.oibvh_scene_autotune(None, 0, 1, None) == N.ERR_ARG
    assert L.oibvh_scene_capture_frame(None, 0, 1, 1, None, None, None) == N.ERR_ARG
    assert L.oibvh_tree_set_morton_bits(None, 63) == N.ERR_ARG
    # the allocation-free detect
    n = ctypes.c_uint32()
    assert L.oibvh_pair_detect_noalloc(None, None, 0, None, 0, ctypes.byref(n), None) == N.ERR_ARG
    # a misaligned output buffer is refused before either handle is read (the
    # handles here are never dereferenced)
    fake = ctypes.c_void_p(64)
    assert L.oibvh_pair_detect_noalloc(fake, fake, 0, ctypes.c_void_p(0x1008), 16, ctypes.byref(n), None) == N.ERR_ARG
    assert b"16-byte aligned" in L.oibvh_last_error()
