"""ORACLE — test infrastructure only.

ctypes bindings for two CPU checkers:

* ``Port``: the plain-C restatement in oracle/oibvh_oracle.c, compiled here
  with gcc (``build_port``) into oracle/_build/liboibvh_oracle.so. It travels
  everywhere and is the checker on the GPU host.
* ``Reference``: the reference's own CPU path compiled from its sources into
  oracle/_ref/libref_cpu.so by oracle/build_ref.sh. It exists only where the
  reference checkout exists; it pins the port and generated the golden
  fixtures under tests/golden/.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module. The product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SRC = os.path.join(HERE, "oibvh_oracle.c")
PORT_LIB = os.path.join(HERE, "_build", "liboibvh_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_cpu.so")
REF_GPU_LIB = os.path.join(HERE, "_ref", "libref_gpu.so")

_u32p = ctypes.POINTER(ctypes.c_uint32)
_f32p = ctypes.POINTER(ctypes.c_float)
_i64p = ctypes.POINTER(ctypes.c_int64)
_lock = threading.Lock()


def build_port(force: bool = False) -> str:
    """Compile the C restatement (gcc, -O2, no FP contraction)."""
    with _lock:
        if not force and os.path.exists(PORT_LIB) and os.path.getmtime(PORT_LIB) >= os.path.getmtime(PORT_SRC):
            return PORT_LIB
        os.makedirs(os.path.dirname(PORT_LIB), exist_ok=True)
        tmp = PORT_LIB + f".{os.getpid()}.tmp"
        subprocess.check_call(
            ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
             "-Wall", "-o", tmp, PORT_SRC, "-lm"]
        )
        os.replace(tmp, PORT_LIB)
        return PORT_LIB


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(_f32p)


def _u32(a):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return a, a.ctypes.data_as(_u32p)


class Port:
    """The C restatement of the reference CPU path (SimpleBVH + DFS detect +
    triangleIntersect) and of the reference GPU tree layout."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = ctypes.CDLL(build_port())
            lib.oracle_scene_create.restype = ctypes.c_void_p
            lib.oracle_scene_destroy.argtypes = [ctypes.c_void_p]
            lib.oracle_scene_add_mesh.argtypes = [ctypes.c_void_p, _f32p, ctypes.c_uint32, _u32p, ctypes.c_uint32]
            lib.oracle_scene_refit.argtypes = [ctypes.c_void_p, ctypes.c_int, _f32p]
            lib.oracle_scene_detect.argtypes = [ctypes.c_void_p, _u32p, ctypes.c_int, _u32p, ctypes.c_int64, _i64p]
            lib.oracle_scene_detect.restype = ctypes.c_int64
            lib.oracle_scene_detect_f64.argtypes = [ctypes.c_void_p, _u32p, ctypes.c_int, _u32p, ctypes.c_int64]
            lib.oracle_scene_detect_f64.restype = ctypes.c_int64
            lib.oracle_scene_leaf_boxes.argtypes = [ctypes.c_void_p, ctypes.c_int, _f32p]
            lib.oracle_tri_intersect.argtypes = [_f32p] * 6
            lib.oracle_tri_intersect_f64.argtypes = [_f32p] * 6
            lib.oracle_oibvh_size.argtypes = [ctypes.c_uint32]
            lib.oracle_oibvh_size.restype = ctypes.c_uint32
            lib.oracle_oibvh_build.argtypes = [_f32p, ctypes.c_uint32, _u32p, ctypes.c_uint32, _f32p, _u32p, _u32p]
            lib.oracle_oibvh_refit.argtypes = [_f32p, _u32p, ctypes.c_uint32, _f32p]
            lib.oracle_morton_codes.argtypes = [_f32p, ctypes.c_uint32, _u32p, ctypes.c_uint32, _u32p]
            lib.oracle_mesh_aabb.argtypes = [_f32p, ctypes.c_uint32, _f32p]
            cls._lib = lib
        return cls._lib

    # --- scene (reference CPU path) -------------------------------------
    def __init__(self):
        self._h = ctypes.c_void_p(self.lib().oracle_scene_create())
        self._keep = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self.lib().oracle_scene_destroy(h)
            self._h = None

    def add_mesh(self, xyz, tri) -> int:
        x, xp = _f32(xyz)
        t, tp = _u32(tri)
        self._keep.append((x, t))
        mid = self.lib().oracle_scene_add_mesh(self._h, xp, x.shape[0], tp, t.shape[0])
        if mid < 0:
            raise RuntimeError("oracle: add_mesh failed")
        self._keep[-1] = (x, t)
        return mid

    def set_positions(self, mid: int, xyz) -> None:
        x, xp = _f32(xyz)
        old_t = self._keep[mid][1]
        self._keep[mid] = (x, old_t)
        if self.lib().oracle_scene_refit(self._h, mid, xp) != 0:
            raise RuntimeError("oracle: refit failed")

    def detect(self, pairs=None, fp64: bool = False):
        """Returns (hits uint32[n,4] {bvhA,bvhB,triA,triB}, n_candidates)."""
        lib = self.lib()
        if pairs is None:
            pp, npairs = None, 0
            pa = None
        else:
            pa, pp = _u32(np.asarray(pairs, dtype=np.uint32).reshape(-1, 2))
            npairs = pa.shape[0]
        cap = 1 << 16
        while True:
            out = np.empty((cap, 4), dtype=np.uint32)
            ncand = ctypes.c_int64(0)
            if fp64:
                n = lib.oracle_scene_detect_f64(self._h, pp, npairs, out.ctypes.data_as(_u32p), cap)
            else:
                n = lib.oracle_scene_detect(self._h, pp, npairs, out.ctypes.data_as(_u32p), cap, ctypes.byref(ncand))
            if n < 0:
                raise RuntimeError("oracle: detect failed")
            if n <= cap:
                return out[:n].copy(), int(ncand.value)
            cap = int(n)

    def leaf_boxes(self, mid: int) -> np.ndarray:
        nT = self._keep[mid][1].shape[0]
        out = np.empty((nT, 6), dtype=np.float32)
        self.lib().oracle_scene_leaf_boxes(self._h, mid, out.ctypes.data_as(_f32p))
        return out

    # --- stateless helpers ----------------------------------------------
    @classmethod
    def tri_intersect(cls, P1, P2, P3, Q1, Q2, Q3, fp64: bool = False) -> bool:
        args = [_f32(v) for v in (P1, P2, P3, Q1, Q2, Q3)]
        fn = cls.lib().oracle_tri_intersect_f64 if fp64 else cls.lib().oracle_tri_intersect
        return bool(fn(*[a[1] for a in args]))

    @classmethod
    def oibvh_size(cls, n_tri: int) -> int:
        return int(cls.lib().oracle_oibvh_size(n_tri))

    @classmethod
    def oibvh_build(cls, xyz, tri):
        """Reference GPU build restated: (aabbs float32[size,6], sorted faces, perm)."""
        x, xp = _f32(xyz)
        t, tp = _u32(tri)
        size = cls.oibvh_size(t.shape[0])
        aabbs = np.empty((size, 6), dtype=np.float32)
        st = np.empty_like(t)
        perm = np.empty(t.shape[0], dtype=np.uint32)
        rc = cls.lib().oracle_oibvh_build(xp, x.shape[0], tp, t.shape[0], aabbs.ctypes.data_as(_f32p),
                                          st.ctypes.data_as(_u32p), perm.ctypes.data_as(_u32p))
        if rc != 0:
            raise RuntimeError(f"oracle: oibvh_build failed ({rc})")
        return aabbs, st, perm

    @classmethod
    def oibvh_refit(cls, xyz, sorted_tri):
        x, xp = _f32(xyz)
        t, tp = _u32(sorted_tri)
        aabbs = np.empty((cls.oibvh_size(t.shape[0]), 6), dtype=np.float32)
        if cls.lib().oracle_oibvh_refit(xp, tp, t.shape[0], aabbs.ctypes.data_as(_f32p)) != 0:
            raise RuntimeError("oracle: oibvh_refit failed")
        return aabbs

    @classmethod
    def morton_codes(cls, xyz, tri) -> np.ndarray:
        x, xp = _f32(xyz)
        t, tp = _u32(tri)
        out = np.empty(t.shape[0], dtype=np.uint32)
        cls.lib().oracle_morton_codes(xp, x.shape[0], tp, t.shape[0], out.ctypes.data_as(_u32p))
        return out


class Reference:
    """The reference's own CPU path (oracle/_ref/libref_cpu.so), where built."""

    _lib = None

    @classmethod
    def available(cls) -> bool:
        try:
            cls.lib()
            return True
        except OSError:
            return False

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = ctypes.CDLL(REF_LIB)
            lib.ref_scene_create.restype = ctypes.c_void_p
            lib.ref_scene_destroy.argtypes = [ctypes.c_void_p]
            lib.ref_scene_add_mesh.argtypes = [ctypes.c_void_p, _f32p, ctypes.c_uint32, _u32p, ctypes.c_uint32]
            lib.ref_scene_set_positions.argtypes = [ctypes.c_void_p, ctypes.c_int, _f32p]
            lib.ref_scene_detect.argtypes = [ctypes.c_void_p, _u32p, ctypes.c_int, _u32p, ctypes.c_longlong,
                                             ctypes.POINTER(ctypes.c_longlong)]
            lib.ref_scene_detect.restype = ctypes.c_longlong
            lib.ref_scene_leaf_boxes.argtypes = [ctypes.c_void_p, ctypes.c_int, _f32p]
            lib.ref_tri_intersect.argtypes = [_f32p] * 6
            cls._lib = lib
        return cls._lib

    def __init__(self):
        self._h = ctypes.c_void_p(self.lib().ref_scene_create())
        self._nt = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self.lib().ref_scene_destroy(h)
            self._h = None

    def add_mesh(self, xyz, tri) -> int:
        x, xp = _f32(xyz)
        t, tp = _u32(tri)
        self._nt.append(t.shape[0])
        return self.lib().ref_scene_add_mesh(self._h, xp, x.shape[0], tp, t.shape[0])

    def set_positions(self, mid: int, xyz) -> None:
        x, xp = _f32(xyz)
        if self.lib().ref_scene_set_positions(self._h, mid, xp) != 0:
            raise RuntimeError("reference: set_positions failed")

    def detect(self, pairs=None):
        lib = self.lib()
        if pairs is None:
            pp, npairs = None, 0
        else:
            pa, pp = _u32(np.asarray(pairs, dtype=np.uint32).reshape(-1, 2))
            npairs = pa.shape[0]
        cap = 1 << 16
        while True:
            out = np.empty((cap, 4), dtype=np.uint32)
            ncand = ctypes.c_longlong(0)
            n = lib.ref_scene_detect(self._h, pp, npairs, out.ctypes.data_as(_u32p), cap, ctypes.byref(ncand))
            if n <= cap:
                return out[:n].copy(), int(ncand.value)
            cap = int(n)

    def leaf_boxes(self, mid: int) -> np.ndarray:
        out = np.empty((self._nt[mid], 6), dtype=np.float32)
        self.lib().ref_scene_leaf_boxes(self._h, mid, out.ctypes.data_as(_f32p))
        return out

    @classmethod
    def tri_intersect(cls, P1, P2, P3, Q1, Q2, Q3) -> bool:
        args = [_f32(v) for v in (P1, P2, P3, Q1, Q2, Q3)]
        return bool(cls.lib().ref_tri_intersect(*[a[1] for a in args]))


class RefGPU:
    """The reference's own GPU kernels (src/cuda/oibvh.cu and src/cuda/collide.cu,
    compiled unmodified by build_ref.sh into oracle/_ref/libref_gpu.so) driven
    by the headless host sequence of oracle/ref_gpu_harness.cu. A build whose
    construction schedule has a partial block, or a detect whose traversal
    would overflow the reference's fixed buffers, is refused on the host
    before any kernel runs (status UNSAFE_*)."""

    OK, CUDA, UNSAFE_SCHEDULE, UNSAFE_CAPACITY, ARG = 0, -1, -2, -3, -4
    _lib = None

    @classmethod
    def available(cls) -> bool:
        try:
            cls.lib()
            return True
        except OSError:
            return False

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = ctypes.CDLL(REF_GPU_LIB)
            vp = ctypes.c_void_p
            lib.refgpu_tree_create.restype = vp
            lib.refgpu_tree_create.argtypes = [_f32p, ctypes.c_uint32, _u32p, ctypes.c_uint32]
            lib.refgpu_tree_destroy.argtypes = [vp]
            lib.refgpu_tree_build.argtypes = [vp, ctypes.c_int, _f32p]
            lib.refgpu_tree_refit.argtypes = [vp, _f32p, _f32p]
            lib.refgpu_tree_get.argtypes = [vp, _f32p, _u32p]
            lib.refgpu_tree_size.argtypes = [vp]
            lib.refgpu_tree_size.restype = ctypes.c_uint32
            lib.refgpu_detect.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, _u32p,
                                          ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong), _f32p]
            lib.refgpu_detect.restype = ctypes.c_longlong
            cls._lib = lib
        return cls._lib

    class Tree:
        def __init__(self, xyz, tri):
            x, xp = _f32(xyz)
            t, tp = _u32(tri)
            self.n_tri = t.shape[0]
            self._h = ctypes.c_void_p(RefGPU.lib().refgpu_tree_create(xp, x.shape[0], tp, t.shape[0]))
            if not self._h.value:
                raise ValueError("reference GPU tree: needs at least 2 triangles")

        def __del__(self):
            h = getattr(self, "_h", None)
            if h is not None and h.value:
                RefGPU.lib().refgpu_tree_destroy(h)
                self._h = None

        def build(self, construct: bool = True):
            """(status, [whole ms, kernels ms]); UNSAFE_SCHEDULE: sorted faces only."""
            ms = np.zeros(2, dtype=np.float32)
            st = RefGPU.lib().refgpu_tree_build(self._h, int(construct), ms.ctypes.data_as(_f32p))
            return int(st), ms

        def refit(self, xyz):
            x, xp = _f32(xyz)
            ms = np.zeros(2, dtype=np.float32)
            st = RefGPU.lib().refgpu_tree_refit(self._h, xp, ms.ctypes.data_as(_f32p))
            return int(st), ms

        def boxes(self) -> np.ndarray:
            n = RefGPU.lib().refgpu_tree_size(self._h)
            out = np.empty((n, 6), dtype=np.float32)
            RefGPU.lib().refgpu_tree_get(self._h, out.ctypes.data_as(_f32p), None)
            return out

        def sorted_faces(self) -> np.ndarray:
            out = np.empty((self.n_tri, 3), dtype=np.uint32)
            RefGPU.lib().refgpu_tree_get(self._h, None, out.ctypes.data_as(_u32p))
            return out

    @classmethod
    def detect(cls, trees, entry: int = 4, expand: int = 3):
        """(status or hit count, hits uint32[n, 4] {bvhA, bvhB, triA, triB} with
        Morton-order triangle indices, candidate count, [whole, traversal,
        narrow] ms). A negative first value is a refusal or a CUDA error."""
        hs = (ctypes.c_void_p * len(trees))(*[t._h.value for t in trees])
        cap = 1 << 22
        out = np.empty((cap, 4), dtype=np.uint32)
        nc = ctypes.c_longlong(0)
        ms = np.zeros(3, dtype=np.float32)
        n = cls.lib().refgpu_detect(hs, len(trees), entry, expand, out.ctypes.data_as(_u32p), cap, ctypes.byref(nc),
                                    ms.ctypes.data_as(_f32p))
        if n < 0:
            return int(n), None, 0, ms
        return int(n), out[: min(n, cap)].copy(), int(nc.value), ms


def sort_pairs(hits: np.ndarray) -> np.ndarray:
    """Lexicographic order on (bvhA, bvhB, triA, triB)."""
    hits = np.asarray(hits, dtype=np.uint32).reshape(-1, 4)
    if hits.shape[0] == 0:
        return hits
    order = np.lexsort((hits[:, 3], hits[:, 2], hits[:, 1], hits[:, 0]))
    return hits[order]
