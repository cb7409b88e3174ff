"""Python mirror of the reference's tree / scene interface, over the C ABI.

    OibvhTree(mesh)            -> OibvhTree::OibvhTree   (src/cuda/oibvhTree.cu:9-15)
    OibvhTree.copy_of(o, mesh) -> OibvhTree(other, mesh) (src/cuda/oibvhTree.cu:17-33)
    tree.build()               -> OibvhTree::build       (src/cuda/oibvhTree.cu:237-388)
    tree.refit(xyz)            -> OibvhTree::refit       (src/cuda/oibvhTree.cu:193-235)
    tree.getDepth(), getPrimCount()                      (src/cuda/oibvhTree.cu:46-54)
    Scene().addOibvhTree(tree)                           (src/cuda/scene.cu:95-129)
    scene.detectCollision(DeviceType.GPU0, 4, 3)         (src/cuda/scene.cu:157-185)
    scene.getIntTriPairCount()                           (src/cuda/scene.cu:50-53)

Every call goes through liboibvh_gb300.so; errors raise OibvhError with the
library's status code (the reference ignores them).
"""
from __future__ import annotations

import ctypes
import enum

import numpy as np

from . import _native as N
from .meshes import Mesh

__all__ = ["DeviceType", "OibvhTree", "Scene", "Server", "OibvhError"]

OibvhError = N.OibvhError


class DeviceType(enum.IntEnum):
    """include/cuda/scene.cuh:12-24"""

    CPU = -1
    GPU0 = 0
    GPU1 = 1
    GPU2 = 2
    GPU3 = 3
    GPU4 = 4
    GPU5 = 5
    GPU6 = 6
    GPU7 = 7
    GPU8 = 8


def _stream_handle(stream) -> ctypes.c_void_p:
    if stream is None:
        return ctypes.c_void_p(None)
    if isinstance(stream, int):
        return ctypes.c_void_p(stream)
    h = getattr(stream, "cuda_stream", None)  # torch.cuda.Stream
    if h is not None:
        return ctypes.c_void_p(int(h))
    raise TypeError("stream must be None, an int handle or a torch.cuda.Stream")


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


class OibvhTree:
    """An oibvh over one triangle mesh, resident on one GPU."""

    def __init__(self, mesh: Mesh | None = None, *, xyz=None, tri=None, device: int = 0, _handle=None):
        self._h = ctypes.c_void_p(None)
        self._nv = 0
        if _handle is not None:
            self._h = _handle
            return
        if mesh is not None:
            xyz, tri = mesh.xyz, mesh.tri
        x = _f32(xyz).reshape(-1, 3)
        t = np.ascontiguousarray(tri, dtype=np.uint32).reshape(-1, 3)
        h = ctypes.c_void_p()
        N.check(
            N.lib().oibvh_tree_create(
                x.ctypes.data_as(N._f32p), x.shape[0], t.ctypes.data_as(N._u32p), t.shape[0], int(device),
                ctypes.byref(h)),
            "oibvh_tree_create",
        )
        self._h = h
        self._nv = int(x.shape[0])

    @classmethod
    def copy_of(cls, other: "OibvhTree", mesh: Mesh | None = None, *, xyz=None) -> "OibvhTree":
        x = _f32(mesh.xyz if mesh is not None else xyz).reshape(-1, 3)
        h = ctypes.c_void_p()
        N.check(N.lib().oibvh_tree_create_copy(other._h, x.ctypes.data_as(N._f32p), x.shape[0], ctypes.byref(h)),
                "oibvh_tree_create_copy")
        t = cls(_handle=h)
        t._nv = int(x.shape[0])
        return t

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                N.lib().oibvh_tree_destroy(h)
            except Exception:
                pass
            self._h = ctypes.c_void_p(None)

    close = __del__

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def build(self, stream=None) -> None:
        N.check(N.lib().oibvh_tree_build(self._h, _stream_handle(stream)), "oibvh_tree_build")

    def set_morton_bits(self, bits: int) -> None:
        """Key width of the next build: 30 (the reference's) or 63."""
        N.check(N.lib().oibvh_tree_set_morton_bits(self._h, int(bits)), "oibvh_tree_set_morton_bits")

    def morton_bits(self) -> int:
        return int(N.lib().oibvh_tree_get_morton_bits(self._h))

    def refit(self, xyz=None, stream=None) -> None:
        """Refit to host positions `xyz` (float32[V,3]), or to the positions
        already held when None. Stream-ordered."""
        if xyz is None:
            N.check(N.lib().oibvh_tree_refit(self._h, None, _stream_handle(stream)), "oibvh_tree_refit")
            return
        x = _f32(xyz)
        if x.size != 3 * self.vertex_count:
            raise ValueError("refit positions must be float32[V,3]")
        N.check(N.lib().oibvh_tree_refit(self._h, x.ctypes.data_as(N._f32p), _stream_handle(stream)),
                "oibvh_tree_refit")
        self._keep = x  # pageable source: copied before the call returns, kept for safety

    def refit_device(self, d_xyz_ptr: int, stream=None) -> None:
        """Refit to positions in device memory (a raw pointer, e.g. tensor.data_ptr())."""
        N.check(N.lib().oibvh_tree_refit_device(self._h, ctypes.c_void_p(int(d_xyz_ptr)), _stream_handle(stream)),
                "oibvh_tree_refit_device")

    def set_positions(self, xyz, stream=None) -> None:
        """Host positions for the next refit (copied, stream-ordered), no refit."""
        x = _f32(xyz)
        if x.size != 3 * self.vertex_count:
            raise ValueError("positions must be float32[V,3]")
        N.check(N.lib().oibvh_tree_set_positions(self._h, x.ctypes.data_as(N._f32p), _stream_handle(stream)),
                "oibvh_tree_set_positions")
        self._keep = x

    def set_positions_device(self, d_xyz_ptr: int, stream=None) -> None:
        """Device xyz positions (raw pointer) for the next refit, converted, no refit."""
        N.check(N.lib().oibvh_tree_set_positions_device(self._h, ctypes.c_void_p(int(d_xyz_ptr)),
                                                         _stream_handle(stream)), "oibvh_tree_set_positions_device")

    def set_positions4_device(self, d_xyzw_ptr: int) -> None:
        """Device xyzw positions (16 B per vertex, 16-B aligned, the caller's vertex
        order), kept by reference: every following refit reads them."""
        N.check(N.lib().oibvh_tree_set_positions4_device(self._h, ctypes.c_void_p(int(d_xyzw_ptr))),
                "oibvh_tree_set_positions4_device")

    # reference accessors
    def getDepth(self) -> int:
        return int(N.lib().oibvh_tree_get_depth(self._h))

    def getPrimCount(self) -> int:
        return int(N.lib().oibvh_tree_get_prim_count(self._h))

    @property
    def size(self) -> int:
        return int(N.lib().oibvh_tree_get_size(self._h))

    @property
    def vertex_count(self) -> int:
        return self._nv

    def aabb_tree(self) -> np.ndarray:
        """m_aabbTree: float32[size, 6] (min xyz, max xyz), level-ordered."""
        out = np.empty((self.size, 6), dtype=np.float32)
        N.check(N.lib().oibvh_tree_get_aabbs(self._h, out.ctypes.data_as(N._f32p), out.shape[0]),
                "oibvh_tree_get_aabbs")
        return out

    def sorted_faces(self) -> tuple[np.ndarray, np.ndarray]:
        n = self.getPrimCount()
        f = np.empty((n, 3), dtype=np.uint32)
        p = np.empty(n, dtype=np.uint32)
        N.check(N.lib().oibvh_tree_get_sorted_faces(self._h, f.ctypes.data_as(N._u32p), p.ctypes.data_as(N._u32p), n),
                "oibvh_tree_get_sorted_faces")
        return f, p


class Scene:
    """A set of trees tested pairwise on one GPU."""

    def __init__(self, device: int = 0):
        h = ctypes.c_void_p()
        N.check(N.lib().oibvh_scene_create(int(device), ctypes.byref(h)), "oibvh_scene_create")
        self._h = h
        self._trees = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                N.lib().oibvh_scene_destroy(h)
            except Exception:
                pass
            self._h = ctypes.c_void_p(None)

    close = __del__

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def addOibvhTree(self, tree: OibvhTree) -> int:
        i = ctypes.c_uint32()
        N.check(N.lib().oibvh_scene_add_tree(self._h, tree.handle, ctypes.byref(i)), "oibvh_scene_add_tree")
        self._trees.append(tree)
        return int(i.value)

    def set_pairs(self, pairs=None) -> None:
        if pairs is None:
            N.check(N.lib().oibvh_scene_set_pairs(self._h, None, 0), "oibvh_scene_set_pairs")
            return
        p = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
        N.check(N.lib().oibvh_scene_set_pairs(self._h, p.ctypes.data_as(N._u32p), p.shape[0]),
                "oibvh_scene_set_pairs")

    def detectCollision(self, deviceType: int = DeviceType.GPU0, entryLevel: int = 0, expandLevels: int = 1,
                        stream=None) -> None:
        N.check(N.lib().oibvh_scene_detect(self._h, int(deviceType), int(entryLevel), int(expandLevels),
                                           _stream_handle(stream)), "oibvh_scene_detect")

    def broad(self, deviceType: int = DeviceType.GPU0, entryLevel: int = 0, expandLevels: int = 1,
              stream=None) -> None:
        N.check(N.lib().oibvh_scene_broad(self._h, int(deviceType), int(entryLevel), int(expandLevels),
                                          _stream_handle(stream)), "oibvh_scene_broad")

    def narrow(self, stream=None) -> None:
        N.check(N.lib().oibvh_scene_narrow(self._h, _stream_handle(stream)), "oibvh_scene_narrow")

    def refit(self, stream=None) -> None:
        """Refit every tree of the scene in one launch (to the positions set last)."""
        N.check(N.lib().oibvh_scene_refit(self._h, _stream_handle(stream)), "oibvh_scene_refit")

    def build(self, stream=None) -> None:
        """Build every tree of the scene, one launch per build stage."""
        N.check(N.lib().oibvh_scene_build(self._h, _stream_handle(stream)), "oibvh_scene_build")

    def transform(self, d_rest_xyzw_ptr: int, d_mats_ptr: int, stream=None) -> None:
        """Tree i's positions = M_i * rest_i (packed xyzw rest positions, 12 floats per matrix)."""
        N.check(N.lib().oibvh_scene_transform(self._h, ctypes.c_void_p(int(d_rest_xyzw_ptr)),
                                              ctypes.c_void_p(int(d_mats_ptr)), _stream_handle(stream)),
                "oibvh_scene_transform")

    def set_tuning(self, **kw) -> None:
        t = N.Tuning()
        N.check(N.lib().oibvh_scene_get_tuning(self._h, ctypes.byref(t)), "oibvh_scene_get_tuning")
        for k, v in kw.items():
            setattr(t, k, int(v))
        N.check(N.lib().oibvh_scene_set_tuning(self._h, ctypes.byref(t)), "oibvh_scene_set_tuning")

    def tuning(self) -> dict:
        t = N.Tuning()
        N.check(N.lib().oibvh_scene_get_tuning(self._h, ctypes.byref(t)), "oibvh_scene_get_tuning")
        return {k: int(getattr(t, k)) for k, _ in N.Tuning._fields_}

    def autotune(self, entryLevel: int = 0, reps: int = 3) -> dict:
        t = N.Tuning()
        N.check(N.lib().oibvh_scene_autotune(self._h, int(entryLevel), int(reps), ctypes.byref(t)),
                "oibvh_scene_autotune")
        return {k: int(getattr(t, k)) for k, _ in N.Tuning._fields_}

    def capture_frame(self, entryLevel: int = 0, expandLevels: int = 1, refit: bool = True,
                      d_rest_xyzw_ptr: int | None = None, d_mats_ptr: int | None = None, stream=None) -> None:
        r = ctypes.c_void_p(int(d_rest_xyzw_ptr)) if d_rest_xyzw_ptr else ctypes.c_void_p(None)
        m = ctypes.c_void_p(int(d_mats_ptr)) if d_mats_ptr else ctypes.c_void_p(None)
        N.check(N.lib().oibvh_scene_capture_frame(self._h, int(entryLevel), int(expandLevels), int(bool(refit)), r, m,
                                                  _stream_handle(stream)), "oibvh_scene_capture_frame")

    def launch_frame(self, stream=None) -> None:
        N.check(N.lib().oibvh_scene_launch_frame(self._h, _stream_handle(stream)), "oibvh_scene_launch_frame")

    def finish_frame(self, stream=None) -> None:
        N.check(N.lib().oibvh_scene_finish_frame(self._h, _stream_handle(stream)), "oibvh_scene_finish_frame")

    def profile_frame(self, stream=None) -> dict:
        """One frame stage by stage with CUDA events between the stages:
        device milliseconds of transform, refit, start (start front + top
        walk), walk (every walk round) and narrow; the results are the frame's."""
        p = N.FrameProfile()
        N.check(N.lib().oibvh_scene_profile_frame(self._h, _stream_handle(stream), ctypes.byref(p)),
                "oibvh_scene_profile_frame")
        return {k: (float(getattr(p, k)) if k.endswith("_ms") else int(getattr(p, k))) for k, _ in p._fields_}

    def getIntTriPairCount(self) -> int:
        return int(N.lib().oibvh_scene_get_int_tri_pair_count(self._h))

    def candidate_count(self) -> int:
        return int(N.lib().oibvh_scene_get_candidate_count(self._h))

    def int_tri_pairs(self, sort: bool = True) -> np.ndarray:
        """uint32[n, 4] records {bvhA, bvhB, triA, triB} with original face indices."""
        n = ctypes.c_uint64()
        cnt = self.getIntTriPairCount()
        out = np.empty((max(cnt, 1), 4), dtype=np.uint32)
        N.check(N.lib().oibvh_scene_get_int_tri_pairs(self._h, out.ctypes.data_as(N._u32p), cnt, ctypes.byref(n)),
                "oibvh_scene_get_int_tri_pairs")
        out = out[: int(n.value)]
        if sort and out.shape[0]:
            out = out[np.lexsort((out[:, 3], out[:, 2], out[:, 1], out[:, 0]))]
        return out

    def candidates(self) -> np.ndarray:
        n = ctypes.c_uint64()
        cnt = self.candidate_count()
        out = np.empty((max(cnt, 1), 4), dtype=np.uint32)
        N.check(N.lib().oibvh_scene_get_candidates(self._h, out.ctypes.data_as(N._u32p), cnt, ctypes.byref(n)),
                "oibvh_scene_get_candidates")
        return out[: int(n.value)]

    def set_queue_capacity(self, front: int = 0, candidates: int = 0, hits: int = 0) -> None:
        N.check(N.lib().oibvh_scene_set_queue_capacity(self._h, int(front), int(candidates), int(hits)),
                "oibvh_scene_set_queue_capacity")

    def set_precision(self, mode: int) -> None:
        """N.PRECISION_FP32 (the reference's float test) or
        N.PRECISION_FP64_FILTERED (float test, undecided axes again in FP64)."""
        N.check(N.lib().oibvh_scene_set_precision(self._h, int(mode)), "oibvh_scene_set_precision")

    def precision(self) -> int:
        return int(N.lib().oibvh_scene_get_precision(self._h))

    def stats(self) -> dict:
        st = N.DetectStats()
        N.check(N.lib().oibvh_scene_get_stats(self._h, ctypes.byref(st)), "oibvh_scene_get_stats")
        return {k: int(getattr(st, k)) for k, _ in N.DetectStats._fields_}


class Server:
    """Continuous-batching request loop over a pool of resident meshes
    (oibvh_server_* in include/oibvh_gb300.h). A query is (mesh A, mesh B,
    3x4 rigid transform of B); its result is B-transformed against A at rest.

        srv = Server(memory_budget=8 << 30, max_batch=256, lanes=4)
        ids = [srv.add_mesh(t) for t in trees]   # built OibvhTree objects
        srv.start()
        t = srv.submit(ids[0], ids[1], mat12)
        info = srv.wait(t); pairs = srv.pairs(t); srv.release(t)
    """

    def __init__(self, device: int = 0, memory_budget: int = 1 << 30, max_batch: int = 256, lanes: int = 4):
        h = ctypes.c_void_p()
        N.check(N.lib().oibvh_server_create(int(device), int(memory_budget), int(max_batch), int(lanes),
                                            ctypes.byref(h)), "oibvh_server_create")
        self._h = h
        self._trees = []  # the pool trees must outlive the server

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            N.lib().oibvh_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_entry_level(self, level: int) -> None:
        N.check(N.lib().oibvh_server_set_entry_level(self._h, int(level)), "oibvh_server_set_entry_level")

    def set_queue_capacity(self, front: int = 0, hits: int = 0) -> None:
        N.check(N.lib().oibvh_server_set_queue_capacity(self._h, int(front), int(hits)),
                "oibvh_server_set_queue_capacity")

    def set_batch_cost(self, max_triangles: int) -> None:
        N.check(N.lib().oibvh_server_set_batch_cost(self._h, int(max_triangles)), "oibvh_server_set_batch_cost")

    def add_mesh(self, tree: "OibvhTree") -> int:
        i = ctypes.c_uint32()
        N.check(N.lib().oibvh_server_add_mesh(self._h, tree.handle, ctypes.byref(i)), "oibvh_server_add_mesh")
        self._trees.append(tree)
        return int(i.value)

    def start(self) -> None:
        N.check(N.lib().oibvh_server_start(self._h), "oibvh_server_start")

    def submit(self, mesh_a: int, mesh_b: int, mat_b) -> int:
        m = np.ascontiguousarray(np.asarray(mat_b, dtype=np.float32).reshape(12))
        t = ctypes.c_uint64()
        N.check(N.lib().oibvh_server_submit(self._h, int(mesh_a), int(mesh_b), m.ctypes.data_as(N._f32p),
                                            ctypes.byref(t)), "oibvh_server_submit")
        return int(t.value)

    def wait(self, ticket: int, timeout_ms: int = 60000) -> dict:
        r = N.QueryResult()
        N.check(N.lib().oibvh_server_wait(self._h, int(ticket), int(timeout_ms), ctypes.byref(r)), "oibvh_server_wait")
        return {k: getattr(r, k) for k, _ in N.QueryResult._fields_}

    def pairs(self, ticket: int) -> np.ndarray:
        """uint32[n, 2] (triA, triB) with original face indices, sorted."""
        n = ctypes.c_uint64()
        N.check(N.lib().oibvh_server_get_pairs(self._h, int(ticket), None, 0, ctypes.byref(n)),
                "oibvh_server_get_pairs")
        out = np.empty((max(int(n.value), 1), 2), dtype=np.uint32)
        N.check(N.lib().oibvh_server_get_pairs(self._h, int(ticket), out.ctypes.data_as(N._u32p), int(n.value),
                                               ctypes.byref(n)), "oibvh_server_get_pairs")
        out = out[: int(n.value)]
        if out.shape[0]:
            out = out[np.lexsort((out[:, 1], out[:, 0]))]
        return out

    def release(self, ticket: int) -> None:
        N.check(N.lib().oibvh_server_release(self._h, int(ticket)), "oibvh_server_release")

    def stats(self) -> dict:
        st = N.ServerStats()
        N.check(N.lib().oibvh_server_get_stats(self._h, ctypes.byref(st)), "oibvh_server_get_stats")
        return {k: int(getattr(st, k)) for k, _ in N.ServerStats._fields_}
