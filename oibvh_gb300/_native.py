"""ctypes binding of the C ABI in include/oibvh_gb300.h.

The CUDA library is built in-tree (oibvh_gb300/_lib/liboibvh_gb300.so, see
build.py). There is no fallback: if the library is missing or fails to load,
``lib()`` raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_u32p = ctypes.POINTER(ctypes.c_uint32)
_f32p = ctypes.POINTER(ctypes.c_float)
_vp = ctypes.c_void_p
_u32 = ctypes.c_uint32
_u64 = ctypes.c_uint64

OK = 0
ERR_ARG = 1
ERR_OOM = 2
ERR_CUDA = 3
ERR_OVERFLOW = 4
ERR_STATE = 5
ERR_UNSUPPORTED = 6
ERR_TIMEOUT = 7
PRECISION_FP32 = 0
PRECISION_FP64_FILTERED = 1
QUERY_QUEUED, QUERY_RUNNING, QUERY_DONE, QUERY_FAILED = 0, 1, 2, 3

DEVICE_CPU = -1


class DetectStats(ctypes.Structure):
    _fields_ = [
        ("passes", ctypes.c_uint32),
        ("steps", ctypes.c_uint32),
        ("retries", ctypes.c_uint32),
        ("frame_redos", ctypes.c_uint32),
        ("nodes_tested", ctypes.c_uint64),
        ("candidates", ctypes.c_uint64),
        ("hits", ctypes.c_uint64),
        ("front_peak", ctypes.c_uint64),
        ("fp64_axes", ctypes.c_uint64),
        ("fp64_candidates", ctypes.c_uint64),
        ("fp32_disagreements", ctypes.c_uint64),
        ("bounded_candidates", ctypes.c_uint64),
    ]


class QueryResult(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int),
        ("error", ctypes.c_int),
        ("lane", ctypes.c_uint32),
        ("batch_size", ctypes.c_uint32),
        ("n_pairs", ctypes.c_uint64),
        ("queue_us", ctypes.c_double),
        ("service_us", ctypes.c_double),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in (
        "submitted", "completed", "failed", "batches", "max_batch_seen", "redos", "candidates", "hits",
        "arena_bytes", "arena_used_bytes", "arena_peak_bytes", "queued")]


class FrameProfile(ctypes.Structure):
    _fields_ = [
        ("transform_ms", ctypes.c_float),
        ("refit_ms", ctypes.c_float),
        ("start_ms", ctypes.c_float),
        ("walk_ms", ctypes.c_float),
        ("narrow_ms", ctypes.c_float),
        ("walk_rounds", ctypes.c_uint32),
        ("kernels", ctypes.c_uint32),
    ]


class Tuning(ctypes.Structure):
    _fields_ = [
        ("start_pairs_log2", ctypes.c_uint32),
        ("handoff", ctypes.c_uint32),
        ("walk_blocks_per_sm", ctypes.c_uint32),
        ("front_capacity", ctypes.c_uint32),
        ("hit_capacity", ctypes.c_uint32),
        ("walk_front", ctypes.c_uint32),
        ("refit_group_log2", ctypes.c_uint32),
        ("descend_ratio", ctypes.c_uint32),
        ("claim_min", ctypes.c_uint32),
    ]


# (name, restype, argtypes) for every symbol of include/oibvh_gb300.h
SIGNATURES = [
    ("oibvh_status_string", ctypes.c_char_p, [ctypes.c_int]),
    ("oibvh_last_error", ctypes.c_char_p, []),
    ("oibvh_version", ctypes.c_int, []),
    ("oibvh_get_launch_count", _u64, []),
    ("oibvh_debug_fail_alloc_after", ctypes.c_int, [ctypes.c_int64]),
    ("oibvh_debug_alloc_attempts", _u64, []),
    ("oibvh_tree_create", ctypes.c_int, [_f32p, _u32, _u32p, _u32, ctypes.c_int, ctypes.POINTER(_vp)]),
    ("oibvh_tree_create_copy", ctypes.c_int, [_vp, _f32p, _u32, ctypes.POINTER(_vp)]),
    ("oibvh_tree_build", ctypes.c_int, [_vp, _vp]),
    ("oibvh_tree_refit", ctypes.c_int, [_vp, _f32p, _vp]),
    ("oibvh_tree_refit_device", ctypes.c_int, [_vp, _vp, _vp]),
    ("oibvh_tree_set_positions", ctypes.c_int, [_vp, _f32p, _vp]),
    ("oibvh_tree_set_positions_device", ctypes.c_int, [_vp, _vp, _vp]),
    ("oibvh_tree_set_positions4_device", ctypes.c_int, [_vp, _vp]),
    ("oibvh_tree_set_morton_bits", ctypes.c_int, [_vp, _u32]),
    ("oibvh_tree_get_morton_bits", _u32, [_vp]),
    ("oibvh_tree_get_depth", _u32, [_vp]),
    ("oibvh_tree_get_prim_count", _u32, [_vp]),
    ("oibvh_tree_get_size", _u32, [_vp]),
    ("oibvh_tree_get_aabbs", ctypes.c_int, [_vp, _f32p, _u64]),
    ("oibvh_tree_get_sorted_faces", ctypes.c_int, [_vp, _u32p, _u32p, _u64]),
    ("oibvh_tree_destroy", ctypes.c_int, [_vp]),
    ("oibvh_scene_create", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_vp)]),
    ("oibvh_scene_add_tree", ctypes.c_int, [_vp, _vp, _u32p]),
    ("oibvh_scene_set_pairs", ctypes.c_int, [_vp, _u32p, _u32]),
    ("oibvh_scene_detect", ctypes.c_int, [_vp, ctypes.c_int, _u32, _u32, _vp]),
    ("oibvh_scene_broad", ctypes.c_int, [_vp, ctypes.c_int, _u32, _u32, _vp]),
    ("oibvh_scene_narrow", ctypes.c_int, [_vp, _vp]),
    ("oibvh_scene_refit", ctypes.c_int, [_vp, _vp]),
    ("oibvh_scene_build", ctypes.c_int, [_vp, _vp]),
    ("oibvh_scene_transform", ctypes.c_int, [_vp, _vp, _vp, _vp]),
    ("oibvh_scene_set_tuning", ctypes.c_int, [_vp, ctypes.POINTER(Tuning)]),
    ("oibvh_scene_get_tuning", ctypes.c_int, [_vp, ctypes.POINTER(Tuning)]),
    ("oibvh_scene_autotune", ctypes.c_int, [_vp, _u32, _u32, ctypes.POINTER(Tuning)]),
    ("oibvh_scene_capture_frame", ctypes.c_int, [_vp, _u32, _u32, ctypes.c_int, _vp, _vp, _vp]),
    ("oibvh_scene_launch_frame", ctypes.c_int, [_vp, _vp]),
    ("oibvh_scene_finish_frame", ctypes.c_int, [_vp, _vp]),
    ("oibvh_scene_get_int_tri_pair_count", _u32, [_vp]),
    ("oibvh_scene_get_candidate_count", _u64, [_vp]),
    ("oibvh_scene_get_int_tri_pairs", ctypes.c_int, [_vp, _u32p, _u64, ctypes.POINTER(_u64)]),
    ("oibvh_scene_get_candidates", ctypes.c_int, [_vp, _u32p, _u64, ctypes.POINTER(_u64)]),
    ("oibvh_scene_set_queue_capacity", ctypes.c_int, [_vp, _u32, _u32, _u32]),
    ("oibvh_scene_set_precision", ctypes.c_int, [_vp, ctypes.c_int]),
    ("oibvh_scene_get_precision", ctypes.c_int, [_vp]),
    ("oibvh_scene_get_stats", ctypes.c_int, [_vp, ctypes.POINTER(DetectStats)]),
    ("oibvh_scene_profile_frame", ctypes.c_int, [_vp, _vp, ctypes.POINTER(FrameProfile)]),
    ("oibvh_scene_destroy", ctypes.c_int, [_vp]),
    ("oibvh_pair_detect_noalloc", ctypes.c_int, [_vp, _vp, _u32, _vp, _u32, _u32p, _vp]),
    ("oibvh_server_create", ctypes.c_int, [ctypes.c_int, _u64, _u32, _u32, ctypes.POINTER(_vp)]),
    ("oibvh_server_set_entry_level", ctypes.c_int, [_vp, _u32]),
    ("oibvh_server_set_queue_capacity", ctypes.c_int, [_vp, _u32, _u32]),
    ("oibvh_server_set_batch_cost", ctypes.c_int, [_vp, _u64]),
    ("oibvh_server_add_mesh", ctypes.c_int, [_vp, _vp, _u32p]),
    ("oibvh_server_start", ctypes.c_int, [_vp]),
    ("oibvh_server_submit", ctypes.c_int, [_vp, _u32, _u32, _f32p, ctypes.POINTER(_u64)]),
    ("oibvh_server_wait", ctypes.c_int, [_vp, _u64, _u32, ctypes.POINTER(QueryResult)]),
    ("oibvh_server_get_pairs", ctypes.c_int, [_vp, _u64, _u32p, _u64, ctypes.POINTER(_u64)]),
    ("oibvh_server_release", ctypes.c_int, [_vp, _u64]),
    ("oibvh_server_get_stats", ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)]),
    ("oibvh_server_destroy", ctypes.c_int, [_vp]),
]

_lib = None
_lock = threading.Lock()


class OibvhError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status: int, func: str, detail: str):
        self.status = status
        self.func = func
        super().__init__(f"{func} failed: {status_string(status)} ({status}): {detail}")


def lib_path() -> str:
    return _build.LIB


def load(path: str | None = None, auto_build: bool = False):
    """Load the library (build it first when auto_build and it is stale)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or lib_path()
        if auto_build and not _build.up_to_date():
            _build.build()
        if not os.path.exists(p):
            raise RuntimeError(
                f"oibvh_gb300 CUDA library not found at {p}; build it with `python -m oibvh_gb300.build` "
                "(there is no CPU fallback)"
            )
        L = ctypes.CDLL(p)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return _lib


def lib():
    return load(auto_build=os.environ.get("OIBVH_AUTO_BUILD", "1") == "1")


def status_string(status: int) -> str:
    try:
        return lib().oibvh_status_string(status).decode()
    except Exception:  # library not loadable: still give a name
        return {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "queue overflow",
                5: "invalid state", 6: "unsupported", 7: "device wait timed out"}.get(status, "unknown status")


def check(status: int, func: str) -> None:
    if status != OK:
        raise OibvhError(status, func, lib().oibvh_last_error().decode(errors="replace"))
