"""ctypes binding of the C ABI in include/collide_gpu.h (libcollide_gpu.so).

This is plumbing for Python callers (tests, bench, the autograd wrapper): every
call goes straight to the CUDA library. There is no CPU fallback; if the
library cannot be built or loaded, or no CUDA device is usable, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

CG_OK = 0
CG_ERR_INVALID_ARGUMENT, CG_ERR_CUDA, CG_ERR_OUT_OF_MEMORY, CG_ERR_QUEUE_OVERFLOW = -1, -2, -3, -4
CG_ERR_OUTPUT_OVERFLOW, CG_ERR_TIMEOUT, CG_ERR_BAD_TREE, CG_ERR_NOT_FOUND = -5, -6, -7, -8
STATUS = {0: "CG_OK", -1: "CG_ERR_INVALID_ARGUMENT", -2: "CG_ERR_CUDA", -3: "CG_ERR_OUT_OF_MEMORY",
          -4: "CG_ERR_QUEUE_OVERFLOW", -5: "CG_ERR_OUTPUT_OVERFLOW", -6: "CG_ERR_TIMEOUT", -7: "CG_ERR_BAD_TREE",
          -8: "CG_ERR_NOT_FOUND"}
CG_KEEP_LEAF_PAIRS = 1
CG_NO_TRI_PAIRS = 2
CG_TRACE = 4
CG_MID_ONLY = 8
CG_CONTACTS = 16
CG_RECHECK = 32
CG_ROBUST = 64
CG_DFS_ORDER = 128

# Every function the header declares (checked by the CPU tests).
EXPORTS = ["cg_config_default", "cg_create", "cg_destroy", "cg_reconfigure", "cg_get_config", "cg_status_string",
           "cg_last_error", "cg_tree_upload", "cg_tree_free", "cg_relative_matrix", "cg_collide", "cg_collide_async",
           "cg_sync_stats", "cg_read_tri_pairs", "cg_read_leaf_pairs", "cg_device_results", "cg_read_contacts",
           "cg_read_rays", "cg_read_ray_averages",
           "cg_traversal_time_ms", "cg_narrow_time_ms", "cg_read_trace", "cg_graph_capture", "cg_graph_launch",
           "cg_collide_static", "cg_deform", "cg_deform_batch", "cg_tree_refit", "cg_tree_refit_batch",
           "cg_tree_download", "cg_pose", "cg_pose_backward", "cg_energy", "cg_energy_backward",
           "cg_set_host_outputs", "cg_shoot_params_default", "cg_shoot_rays",
           "cg_broad_phase", "cg_collision_frame", "cg_tree_build", "cg_tree_info", "cg_tree_export",
           "cg_frame_callbacks", "cg_tree_save", "cg_tree_load"]
CG_STATIC_MAX_QUERIES = 1024
CG_STATIC_MAX_LEAF_PAIRS = 131072


class CgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class cg_config(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_queries", C.c_uint32), ("max_tri_pairs", C.c_uint64),
                ("max_leaf_pairs", C.c_uint64), ("queue_capacity", C.c_uint32), ("warps_per_block", C.c_uint32),
                ("blocks_per_sm", C.c_uint32), ("stack_entries", C.c_uint32), ("donate_min", C.c_uint32),
                ("leaf_flush", C.c_uint32), ("wait_limit_ms", C.c_uint32), ("pad", C.c_uint32),
                ("max_contacts", C.c_uint64)]


class cg_obb(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("u", C.c_float * 3), ("v", C.c_float * 3), ("w", C.c_float * 3)]


class cg_tree_view(C.Structure):
    _fields_ = [("root_obb", cg_obb), ("node_count", C.c_uint32), ("node_obbs", C.c_void_p),
                ("node_ref", C.c_void_p), ("node_tri_count", C.c_void_p), ("triangle_count", C.c_uint32),
                ("triangles_position", C.c_void_p), ("triangles_normal", C.c_void_p),
                ("triangles_indices", C.c_void_p)]


class cg_mesh_view(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("indices", C.c_void_p),
                ("n_vertices", C.c_uint32), ("n_triangles", C.c_uint32)]


class TreeArrays:
    """A tree's flat layout (cg_tree_export): the reference's node layout
    (OBBtree.h:61-75) with its triangles in leaf order."""

    def __init__(self, root, node_obbs, node_ref, node_cnt, tri_pos, tri_nrm, tri_idx):
        self.root = np.ascontiguousarray(root, np.float32).reshape(12)
        self.node_obbs = np.ascontiguousarray(node_obbs, np.float32).reshape(-1, 2, 12)
        self.node_ref = np.ascontiguousarray(node_ref, np.uint32).reshape(-1, 2)
        self.node_cnt = np.ascontiguousarray(node_cnt, np.uint32).reshape(-1, 2)
        self.tri_pos = np.ascontiguousarray(tri_pos, np.float32).reshape(-1, 9)
        self.tri_nrm = None if tri_nrm is None else np.ascontiguousarray(tri_nrm, np.float32).reshape(-1, 9)
        self.tri_idx = np.ascontiguousarray(tri_idx, np.uint32).reshape(-1, 3)

    def arrays(self) -> dict:
        d = dict(root=self.root, node_obbs=self.node_obbs, node_ref=self.node_ref, node_cnt=self.node_cnt,
                 tri_pos=self.tri_pos, tri_idx=self.tri_idx)
        if self.tri_nrm is not None:
            d["tri_nrm"] = self.tri_nrm
        return d


class cg_deform_view(C.Structure):
    _fields_ = [("n_vertices", C.c_uint32), ("n_targets", C.c_uint32), ("n_groups", C.c_uint32),
                ("n_joints", C.c_uint32), ("vertices", C.c_void_p), ("morph_weights", C.c_void_p),
                ("joints", C.c_void_p), ("weights", C.c_void_p), ("joint_matrices", C.c_void_p),
                ("inverse_bind", C.c_void_p)]


class cg_skeleton_view(C.Structure):
    _fields_ = [("n_bones", C.c_uint32), ("parent", C.c_void_p), ("offsets", C.c_void_p)]


class cg_energy_side(C.Structure):
    _fields_ = [("views", C.c_void_p), ("joint_stride", C.c_uint32), ("target_stride", C.c_uint32),
                ("grad_joint_matrices", C.c_void_p), ("grad_morph_weights", C.c_void_p)]


class cg_shoot_params(C.Structure):
    _fields_ = [("smoothstep_start", C.c_float), ("smoothstep_finish", C.c_float), ("distance_bias", C.c_float)]


class cg_shoot_query(C.Structure):
    _fields_ = [("tree_a", C.c_uint32), ("tree_b", C.c_uint32), ("first_global", C.c_float * 16),
                ("second_global", C.c_float * 16), ("n_first", C.c_uint32), ("n_second", C.c_uint32)]


class cg_static_counts(C.Structure):
    _fields_ = [("tri_pairs", C.c_uint64), ("tri_tests", C.c_uint64), ("leaf_pairs", C.c_uint64),
                ("status", C.c_int32), ("pad", C.c_int32)]


class cg_stats(C.Structure):
    _fields_ = [("node_pairs", C.c_uint64), ("leaf_pairs", C.c_uint64), ("tri_tests", C.c_uint64),
                ("tri_pairs", C.c_uint64), ("fragile", C.c_uint64), ("donations", C.c_uint64), ("warp_steps", C.c_uint64),
                ("contacts", C.c_uint64), ("rays", C.c_uint64), ("status", C.c_int32), ("pad", C.c_int32),
                ("rechecked", C.c_uint64), ("disagreements", C.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


QUERY_DTYPE = np.dtype([("tree_a", "<u4"), ("tree_b", "<u4"), ("relative", "<f4", (16,))])
TRI_PAIR_DTYPE = np.dtype([("query", "<u4"), ("tri_a", "<u4"), ("tri_b", "<u4"), ("source", "<f4", (3,)),
                           ("target", "<f4", (3,))])
LEAF_PAIR_DTYPE = np.dtype([("query", "<u4"), ("offset_a", "<u4"), ("offset_b", "<u4"), ("count_a", "<u2"),
                            ("count_b", "<u2")])
CONTACT_DTYPE = np.dtype([("query", "<u4"), ("side", "<u4"), ("tri", "<u4"), ("mask", "<u4"),
                          ("weighted_avg", "<f4", (3,)), ("weight", "<f4")])
RAY_DTYPE = np.dtype([("query", "<u4"), ("side", "<u4"), ("origin", "<f4", (3,)), ("direction", "<f4", (3,))])
RAY_AVERAGE_DTYPE = np.dtype([("first", "<f4", (3,)), ("second", "<f4", (3,)), ("rays_first", "<u4"),
                              ("rays_second", "<u4")])
SHOOT_QUERY_DTYPE = np.dtype([("tree_a", "<u4"), ("tree_b", "<u4"), ("first_global", "<f4", (16,)),
                              ("second_global", "<f4", (16,)), ("n_first", "<u4"), ("n_second", "<u4")])
assert SHOOT_QUERY_DTYPE.itemsize == 144
FRAME_ENTITY_DTYPE = np.dtype([("tree", "<u4"), ("should_callback", "<u4"), ("current_global", "<f4", (16,)),
                               ("previous_global", "<f4", (16,))])
FRAME_RESULT_DTYPE = np.dtype([("first", "<u4"), ("second", "<u4"), ("first_delta", "<f4", (3,)),
                               ("second_delta", "<f4", (3,)), ("query", "<u4"), ("reserved", "<u4")])
FRAME_CALLBACK_DTYPE = np.dtype([("receiver", "<u4"), ("family_entity", "<u4"), ("collide_with", "<u4"),
                                 ("delta", "<f4", (3,))])
assert FRAME_ENTITY_DTYPE.itemsize == 136 and FRAME_RESULT_DTYPE.itemsize == 40
assert FRAME_CALLBACK_DTYPE.itemsize == 24
assert QUERY_DTYPE.itemsize == 72 and TRI_PAIR_DTYPE.itemsize == 36 and LEAF_PAIR_DTYPE.itemsize == 16
assert CONTACT_DTYPE.itemsize == 32 and RAY_DTYPE.itemsize == 32 and RAY_AVERAGE_DTYPE.itemsize == 32

_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Loads (building first if needed) libcollide_gpu.so."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or _build.build()
    lib = C.CDLL(path)
    vp, u32, u64 = C.c_void_p, C.c_uint32, C.c_uint64
    lib.cg_config_default.argtypes = [C.POINTER(cg_config)]
    lib.cg_config_default.restype = None
    lib.cg_create.argtypes = [C.POINTER(cg_config), C.POINTER(vp)]
    lib.cg_destroy.argtypes = [vp]
    lib.cg_reconfigure.argtypes = [vp, C.POINTER(cg_config)]
    lib.cg_get_config.argtypes = [vp, C.POINTER(cg_config)]
    lib.cg_status_string.argtypes = [C.c_int]
    lib.cg_status_string.restype = C.c_char_p
    lib.cg_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    lib.cg_tree_upload.argtypes = [vp, C.POINTER(cg_tree_view), C.POINTER(u32)]
    lib.cg_tree_build.argtypes = [vp, vp, u32, vp]
    lib.cg_tree_info.argtypes = [vp, u32, vp, vp, vp]
    lib.cg_tree_export.argtypes = [vp, u32, vp, vp, vp, vp, vp, vp, vp]
    lib.cg_tree_save.argtypes = [vp, u32, C.c_char_p]
    lib.cg_tree_load.argtypes = [vp, C.c_char_p, C.POINTER(u32)]
    lib.cg_tree_free.argtypes = [vp, u32]
    lib.cg_relative_matrix.argtypes = [vp, vp, vp]
    lib.cg_collide.argtypes = [vp, vp, u32, u32, C.POINTER(cg_stats)]
    lib.cg_collide_async.argtypes = [vp, vp, u32, u32, vp]
    lib.cg_sync_stats.argtypes = [vp, C.POINTER(cg_stats)]
    lib.cg_read_tri_pairs.argtypes = [vp, vp, u64, C.POINTER(u64)]
    lib.cg_read_leaf_pairs.argtypes = [vp, vp, u64, C.POINTER(u64)]
    lib.cg_device_results.argtypes = [vp, C.POINTER(vp), C.POINTER(vp)]
    lib.cg_read_contacts.argtypes = [vp, vp, u64, C.POINTER(u64)]
    lib.cg_read_rays.argtypes = [vp, vp, u64, C.POINTER(u64)]
    lib.cg_read_ray_averages.argtypes = [vp, vp, u64, C.POINTER(u64)]
    lib.cg_traversal_time_ms.argtypes = [vp, C.POINTER(C.c_float)]
    lib.cg_read_trace.argtypes = [vp, u32, vp, u32]
    lib.cg_narrow_time_ms.argtypes = [vp, C.POINTER(C.c_float)]
    lib.cg_graph_capture.argtypes = [vp, vp, u32, u32]
    lib.cg_graph_launch.argtypes = [vp, vp]
    lib.cg_collide_static.argtypes = [vp, vp, u32, vp, u64, vp, vp]
    lib.cg_deform.argtypes = [vp, C.POINTER(cg_deform_view), vp, vp]
    lib.cg_tree_refit.argtypes = [vp, u32, vp, u32, vp]
    lib.cg_deform_batch.argtypes = [vp, vp, vp, u32, vp]
    lib.cg_tree_refit_batch.argtypes = [vp, vp, vp, vp, u32, vp]
    lib.cg_tree_download.argtypes = [vp, u32, vp, vp, u32, vp, u32]
    lib.cg_set_host_outputs.argtypes = [vp, vp, u64, vp, u64, vp, u64]
    lib.cg_broad_phase.argtypes = [vp, vp, vp, vp, u32, vp, vp, u64, C.POINTER(u64)]
    lib.cg_shoot_params_default.argtypes = [C.POINTER(cg_shoot_params)]
    lib.cg_collision_frame.argtypes = [vp, vp, u32, C.POINTER(cg_shoot_params), vp, u64, C.POINTER(u64)]
    lib.cg_frame_callbacks.argtypes = [vp, u64, vp, u32, vp, u32, vp, u64, C.POINTER(u64)]
    lib.cg_shoot_params_default.restype = None
    lib.cg_shoot_rays.argtypes = [vp, vp, u32, vp, u64, C.POINTER(cg_shoot_params), vp]
    lib.cg_pose.argtypes = [vp, C.POINTER(cg_skeleton_view), vp, u32, vp, vp]
    lib.cg_pose_backward.argtypes = [vp, C.POINTER(cg_skeleton_view), vp, vp, vp, u32, vp, vp]
    lib.cg_energy.argtypes = [vp, vp, vp]
    lib.cg_energy_backward.argtypes = [vp, vp, C.POINTER(cg_energy_side), C.POINTER(cg_energy_side), vp]
    _lib = lib
    return lib


def default_config(**over) -> cg_config:
    cfg = cg_config()
    load_library().cg_config_default(C.byref(cfg))
    for k, v in over.items():
        setattr(cfg, k, v)
    return cfg


def relative_matrix(a16, b16) -> np.ndarray:
    a = np.ascontiguousarray(a16, np.float32).reshape(16)
    b = np.ascontiguousarray(b16, np.float32).reshape(16)
    out = np.zeros(16, np.float32)
    rc = load_library().cg_relative_matrix(a.ctypes.data, b.ctypes.data, out.ctypes.data)
    if rc != CG_OK:
        raise CgError(rc, "cg_relative_matrix")
    return out


def frame_callbacks(results: np.ndarray, entity_ids, parent) -> np.ndarray:
    """cg_frame_callbacks (host only): a frame's FRAME_RESULT_DTYPE records
    fanned out to the entities' ancestors; FRAME_CALLBACK_DTYPE, grouped by
    receiver."""
    lib = load_library()
    res = np.ascontiguousarray(results, FRAME_RESULT_DTYPE)
    ids = np.ascontiguousarray(entity_ids, np.uint32)
    par = np.ascontiguousarray(parent, np.uint32)
    cnt = C.c_uint64()
    args = (res.ctypes.data if len(res) else None, len(res), ids.ctypes.data if len(ids) else None, len(ids),
            par.ctypes.data if len(par) else None, len(par))
    rc = lib.cg_frame_callbacks(*args, None, 0, C.byref(cnt))
    if rc not in (0, CG_ERR_OUTPUT_OVERFLOW):
        raise CgError(rc, "cg_frame_callbacks")
    out = np.zeros(max(cnt.value, 1), FRAME_CALLBACK_DTYPE)
    rc = lib.cg_frame_callbacks(*args, out.ctypes.data, len(out), C.byref(cnt))
    if rc != 0:
        raise CgError(rc, "cg_frame_callbacks")
    return out[:cnt.value]


def make_queries(tree_a, tree_b, relative) -> np.ndarray:
    tree_a = np.asarray(tree_a, np.uint32).reshape(-1)
    q = np.zeros(tree_a.size, QUERY_DTYPE)
    q["tree_a"] = tree_a
    q["tree_b"] = np.asarray(tree_b, np.uint32).reshape(-1)
    q["relative"] = np.asarray(relative, np.float32).reshape(-1, 16)
    return q


class Context:
    """One cg_ctx: trees, launch buffers and a CUDA stream on one device."""

    def __init__(self, config: cg_config | None = None, **over):
        self.lib = load_library()
        cfg = config if config is not None else default_config(**over)
        h = C.c_void_p()
        rc = self.lib.cg_create(C.byref(cfg), C.byref(h))
        if rc != CG_OK:
            raise CgError(rc, "cg_create (is a CUDA device available?)")
        self.h = h
        self._trees: dict[int, tuple] = {}

    # -- housekeeping
    def close(self):
        if getattr(self, "h", None):
            self.lib.cg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def last_error(self) -> str:
        buf = C.create_string_buffer(512)
        self.lib.cg_last_error(self.h, buf, 512)
        return buf.value.decode()

    def _check(self, rc: int, what: str):
        if rc != CG_OK:
            raise CgError(rc, f"{what}: {self.last_error()}")

    def config(self) -> cg_config:
        cfg = cg_config()
        self._check(self.lib.cg_get_config(self.h, C.byref(cfg)), "cg_get_config")
        return cfg

    def reconfigure(self, **over):
        cfg = self.config()
        for k, v in over.items():
            setattr(cfg, k, v)
        self._check(self.lib.cg_reconfigure(self.h, C.byref(cfg)), "cg_reconfigure")

    # -- trees
    def upload_tree(self, root, node_obbs, node_ref, node_cnt, tri_pos, tri_nrm=None, tri_idx=None) -> int:
        root = np.ascontiguousarray(root, np.float32).reshape(12)
        node_obbs = np.ascontiguousarray(node_obbs, np.float32).reshape(-1, 2, 12)
        node_ref = np.ascontiguousarray(node_ref, np.uint32).reshape(-1, 2)
        node_cnt = np.ascontiguousarray(node_cnt, np.uint32).reshape(-1, 2)
        tri_pos = np.ascontiguousarray(tri_pos, np.float32).reshape(-1, 9)
        tri_nrm = None if tri_nrm is None else np.ascontiguousarray(tri_nrm, np.float32).reshape(-1, 9)
        tri_idx = None if tri_idx is None else np.ascontiguousarray(tri_idx, np.uint32).reshape(-1, 3)
        v = cg_tree_view()
        for k, name in enumerate(("center", "u", "v", "w")):
            getattr(v.root_obb, name)[:] = root[3 * k:3 * k + 3]
        v.node_count = node_obbs.shape[0]
        v.node_obbs = node_obbs.ctypes.data if node_obbs.size else None
        v.node_ref = node_ref.ctypes.data if node_ref.size else None
        v.node_tri_count = node_cnt.ctypes.data if node_cnt.size else None
        v.triangle_count = tri_pos.shape[0]
        v.triangles_position = tri_pos.ctypes.data if tri_pos.size else None
        v.triangles_normal = None if tri_nrm is None else tri_nrm.ctypes.data
        v.triangles_indices = None if tri_idx is None else tri_idx.ctypes.data
        tid = C.c_uint32()
        self._check(self.lib.cg_tree_upload(self.h, C.byref(v), C.byref(tid)), "cg_tree_upload")
        return tid.value

    def build_trees(self, meshes) -> np.ndarray:
        """cg_tree_build: one tree per mesh (objects with points (V, 3),
        indices (T, 3) and normals (V, 3) or None); their ids."""
        keep, views = [], (cg_mesh_view * max(len(meshes), 1))()
        for k, m in enumerate(meshes):
            pts = np.ascontiguousarray(m.points, np.float32).reshape(-1, 3)
            idx = np.ascontiguousarray(m.indices, np.uint32).reshape(-1, 3)
            nrm = None if getattr(m, "normals", None) is None else np.ascontiguousarray(m.normals, np.float32)
            keep += [pts, idx, nrm]
            views[k].positions = pts.ctypes.data if pts.size else None
            views[k].normals = None if nrm is None else nrm.ctypes.data
            views[k].indices = idx.ctypes.data if idx.size else None
            views[k].n_vertices = len(pts)
            views[k].n_triangles = len(idx)
        ids = np.zeros(max(len(meshes), 1), np.uint32)
        self._check(self.lib.cg_tree_build(self.h, views, len(meshes), ids.ctypes.data), "cg_tree_build")
        return ids[:len(meshes)]

    def tree_info(self, tid: int) -> tuple[int, int, bool]:
        n, t, h = C.c_uint32(), C.c_uint32(), C.c_uint32()
        self._check(self.lib.cg_tree_info(self.h, tid, C.byref(n), C.byref(t), C.byref(h)), "cg_tree_info")
        return n.value, t.value, bool(h.value)

    def export_tree(self, tid: int) -> TreeArrays:
        """cg_tree_export: the tree's whole flat layout."""
        n, t, has_nrm = self.tree_info(tid)
        root = np.zeros(12, np.float32)
        obbs = np.zeros((max(n, 1), 2, 12), np.float32)
        ref = np.zeros((max(n, 1), 2), np.uint32)
        cnt = np.zeros((max(n, 1), 2), np.uint32)
        pos = np.zeros((max(t, 1), 9), np.float32)
        nrm = np.zeros((max(t, 1), 9), np.float32) if has_nrm else None
        idx = np.zeros((max(t, 1), 3), np.uint32)
        self._check(self.lib.cg_tree_export(self.h, tid, root.ctypes.data, obbs.ctypes.data, ref.ctypes.data,
                                            cnt.ctypes.data, pos.ctypes.data,
                                            None if nrm is None else nrm.ctypes.data, idx.ctypes.data),
                    "cg_tree_export")
        return TreeArrays(root, obbs[:n], ref[:n], cnt[:n], pos[:t], None if nrm is None else nrm[:t], idx[:t])

    def save_tree(self, tid: int, path: str):
        """cg_tree_save: the tree cache file."""
        self._check(self.lib.cg_tree_save(self.h, tid, os.fsencode(path)), "cg_tree_save")

    def load_tree(self, path: str) -> int:
        """cg_tree_load: a tree from its cache file; its id."""
        tid = C.c_uint32()
        self._check(self.lib.cg_tree_load(self.h, os.fsencode(path), C.byref(tid)), "cg_tree_load")
        return tid.value

    def upload_flat(self, ft) -> int:
        """Uploads an oracle-style flat tree (attributes root, node_obbs, ...)."""
        return self.upload_tree(ft.root, ft.node_obbs, ft.node_ref, ft.node_cnt, ft.tri_pos, ft.tri_nrm, ft.tri_idx)

    def free_tree(self, tid: int):
        self._check(self.lib.cg_tree_free(self.h, tid), "cg_tree_free")

    # -- collide
    def collide(self, queries: np.ndarray, flags: int = 0, check: bool = True) -> dict:
        q = np.ascontiguousarray(queries, QUERY_DTYPE)
        st = cg_stats()
        rc = self.lib.cg_collide(self.h, q.ctypes.data if q.size else None, q.size, flags, C.byref(st))
        if check:
            self._check(rc, "cg_collide")
        d = st.as_dict()
        d["rc"] = rc
        return d

    def collide_async(self, d_queries_ptr: int, n: int, flags: int = 0, stream: int | None = None):
        self._check(self.lib.cg_collide_async(self.h, d_queries_ptr, n, flags, stream), "cg_collide_async")

    def sync_stats(self, check: bool = True) -> dict:
        st = cg_stats()
        rc = self.lib.cg_sync_stats(self.h, C.byref(st))
        if check:
            self._check(rc, "cg_sync_stats")
        d = st.as_dict()
        d["rc"] = rc
        return d

    def tri_pairs(self, out: np.ndarray | None = None, count: int | None = None) -> np.ndarray:
        """Colliding pairs of the last launch. With `out` (a TRI_PAIR_DTYPE array,
        e.g. a view of pinned memory) and the pair `count` known from the stats,
        the read is a single device-to-host copy into it."""
        n = C.c_uint64()
        if count is None:
            self.lib.cg_read_tri_pairs(self.h, None, 0, C.byref(n))
            count = n.value
        if out is None or len(out) < count:
            out = np.zeros(count, TRI_PAIR_DTYPE)
        rc = self.lib.cg_read_tri_pairs(self.h, out.ctypes.data if count else None, count, C.byref(n))
        self._check(rc, "cg_read_tri_pairs")
        return out[:n.value]

    def leaf_pairs(self) -> np.ndarray:
        n = C.c_uint64()
        self.lib.cg_read_leaf_pairs(self.h, None, 0, C.byref(n))
        out = np.zeros(n.value, LEAF_PAIR_DTYPE)
        rc = self.lib.cg_read_leaf_pairs(self.h, out.ctypes.data if n.value else None, n.value, C.byref(n))
        self._check(rc, "cg_read_leaf_pairs")
        return out

    def _read(self, fn, dtype, out: np.ndarray | None = None, count: int | None = None) -> np.ndarray:
        n = C.c_uint64()
        if count is None:
            self._check(getattr(self.lib, fn)(self.h, None, 0, C.byref(n)), fn)
            count = n.value
        if out is None or len(out) < count:
            out = np.zeros(count, dtype)
        rc = getattr(self.lib, fn)(self.h, out.ctypes.data if count else None, count, C.byref(n))
        self._check(rc, fn)
        return out[:n.value]

    def contacts(self, out: np.ndarray | None = None, count: int | None = None) -> np.ndarray:
        """Per-triangle contacts of the last CG_CONTACTS launch (CONTACT_DTYPE):
        grouped by query, then side, each group in the order of the
        reference's per-triangle map."""
        return self._read("cg_read_contacts", CONTACT_DTYPE, out, count)

    def rays(self, out: np.ndarray | None = None, count: int | None = None) -> np.ndarray:
        """Uncollide rays of the last CG_CONTACTS launch (RAY_DTYPE): grouped by
        query, then side, each group in the reference's order."""
        return self._read("cg_read_rays", RAY_DTYPE, out, count)

    def ray_averages(self, out: np.ndarray | None = None, count: int | None = None) -> np.ndarray:
        """Per query: mean ray origins of both sides (RAY_AVERAGE_DTYPE)."""
        return self._read("cg_read_ray_averages", RAY_AVERAGE_DTYPE, out, count)

    def collide_static(self, d_queries_ptr: int, n: int, d_pairs_ptr: int, pairs_cap: int, d_counts_ptr: int,
                       stream: int | None = None):
        """cg_collide_static: device queries in, pairs and a cg_static_counts
        written to caller-owned device memory on `stream`; nothing allocated."""
        rc = self.lib.cg_collide_static(self.h, d_queries_ptr or None, n, d_pairs_ptr or None, pairs_cap,
                                        d_counts_ptr, stream)
        self._check(rc, "cg_collide_static")

    def deform(self, n_vertices: int, n_targets: int, n_groups: int, n_joints: int, vertices: int,
               morph_weights: int, joints: int, weights: int, joint_matrices: int, inverse_bind: int, out: int,
               stream: int | None = None):
        """cg_deform on device pointers (see cg_deform_view)."""
        v = cg_deform_view(n_vertices, n_targets, n_groups, n_joints, vertices, morph_weights, joints, weights,
                           joint_matrices, inverse_bind)
        self._check(self.lib.cg_deform(self.h, C.byref(v), out, stream), "cg_deform")

    def tree_refit(self, tree_id: int, positions: int, n_positions: int, stream: int | None = None):
        """cg_tree_refit: positions is a device pointer to n_positions float4."""
        self._check(self.lib.cg_tree_refit(self.h, tree_id, positions, n_positions, stream), "cg_tree_refit")

    def deform_batch(self, views: list, outs: list, stream: int | None = None):
        """cg_deform_batch: views are cg_deform_view, outs device pointers."""
        arr = (cg_deform_view * len(views))(*views)
        optr = (C.c_void_p * len(outs))(*outs)
        self._check(self.lib.cg_deform_batch(self.h, arr, optr, len(views), stream), "cg_deform_batch")

    def tree_refit_batch(self, tree_ids, positions, n_positions, stream: int | None = None):
        n = len(tree_ids)
        ids = (C.c_uint32 * n)(*tree_ids)
        pos = (C.c_void_p * n)(*positions)
        cnt = (C.c_uint32 * n)(*n_positions)
        self._check(self.lib.cg_tree_refit_batch(self.h, ids, pos, cnt, n, stream), "cg_tree_refit_batch")

    def tree_download(self, tree_id: int, node_count: int, triangle_count: int):
        """(root (12,), node_obbs (node_count, 2, 12), triangle positions (triangle_count, 9))."""
        root = np.zeros(12, np.float32)
        obbs = np.zeros((max(node_count, 1), 2, 12), np.float32)
        tri = np.zeros((max(triangle_count, 1), 9), np.float32)
        rc = self.lib.cg_tree_download(self.h, tree_id, root.ctypes.data, obbs.ctypes.data if node_count else None,
                                       node_count, tri.ctypes.data if triangle_count else None, triangle_count)
        self._check(rc, "cg_tree_download")
        return root, obbs[:node_count], tri[:triangle_count]

    def set_host_outputs(self, pairs: np.ndarray | None = None, rays: np.ndarray | None = None,
                         averages: np.ndarray | None = None):
        """cg_set_host_outputs on page-locked numpy arrays (e.g. from
        torch.empty(..., pin_memory=True).numpy()) of TRI_PAIR_DTYPE,
        RAY_DTYPE and RAY_AVERAGE_DTYPE; None turns a destination off. The
        arrays must stay alive while set."""
        def arg(a, dt):
            if a is None:
                return None, 0
            assert a.dtype == dt and a.flags.c_contiguous
            return a.ctypes.data, len(a)

        p, r, v = arg(pairs, TRI_PAIR_DTYPE), arg(rays, RAY_DTYPE), arg(averages, RAY_AVERAGE_DTYPE)
        self._check(self.lib.cg_set_host_outputs(self.h, p[0], p[1], r[0], r[1], v[0], v[1]), "cg_set_host_outputs")
        self._host_outputs = (pairs, rays, averages)

    def broad_phase(self, tree_ids, globals_, callback=None, axes=None, cap: int | None = None) -> np.ndarray:
        """cg_broad_phase: (k, 2) [first, second] entity indices (the engine's
        axes unless axes (3, 3))."""
        ids = np.ascontiguousarray(tree_ids, np.uint32)
        n = len(ids)
        g = np.ascontiguousarray(globals_, np.float32).reshape(n, 16)
        cb = None if callback is None else np.ascontiguousarray(callback, np.uint8)
        ax = None if axes is None else np.ascontiguousarray(axes, np.float32).reshape(9)
        cap = n * (n - 1) // 2 if cap is None else cap
        out = np.zeros((max(cap, 1), 2), np.uint32)
        cnt = C.c_uint64()
        rc = self.lib.cg_broad_phase(self.h, ids.ctypes.data if n else None, g.ctypes.data if n else None,
                                     cb.ctypes.data if cb is not None else None, n,
                                     ax.ctypes.data if ax is not None else None, out.ctypes.data, cap, C.byref(cnt))
        self._check(rc, "cg_broad_phase")
        return out[:cnt.value]

    def collision_frame(self, tree_ids, current, previous, callback=None, params: tuple | None = None,
                        cap: int | None = None) -> np.ndarray:
        """cg_collision_frame: one frame of the engine's collision detection
        over n entities (tree ids (n,), current and previous world matrices
        (n, 16), should-callback flags (n,) or all). A FRAME_RESULT_DTYPE array,
        one record per broad pair with rays, in no fixed order."""
        ids = np.ascontiguousarray(tree_ids, np.uint32)
        n = len(ids)
        ent = np.zeros(n, FRAME_ENTITY_DTYPE)
        ent["tree"] = ids
        ent["should_callback"] = 1 if callback is None else np.asarray(callback, np.uint32)
        ent["current_global"] = np.asarray(current, np.float32).reshape(n, 16)
        ent["previous_global"] = np.asarray(previous, np.float32).reshape(n, 16)
        cap = self.config().max_queries if cap is None else cap
        out = np.zeros(max(cap, 1), FRAME_RESULT_DTYPE)
        cnt = C.c_uint64()
        pp = None if params is None else cg_shoot_params(*[float(x) for x in params])
        rc = self.lib.cg_collision_frame(self.h, ent.ctypes.data if n else None, n,
                                         C.byref(pp) if pp is not None else None, out.ctypes.data, cap,
                                         C.byref(cnt))
        self._check(rc, "cg_collision_frame")
        return out[:cnt.value]

    def shoot_rays(self, tree_a, tree_b, first_globals, second_globals, rays_first, rays_second,
                   params: tuple | None = None) -> np.ndarray:
        """cg_shoot_rays for n pairs: tree ids (n,), world matrices (n, 16),
        per pair its rays from the first and from the second entity ((k, 6)
        arrays in the first entity's space); params (start, finish angle in
        radians, bias) or the engine's. The deltas (n, 3)."""
        q, rays = self.pack_shoot(tree_a, tree_b, first_globals, second_globals, rays_first, rays_second)
        return self.shoot_packed(q, rays, params)

    @staticmethod
    def pack_shoot(tree_a, tree_b, first_globals, second_globals, rays_first, rays_second):
        """(SHOOT_QUERY_DTYPE array, (n_rays, 6) float32 rays) for shoot_packed."""
        n = len(tree_a)
        q = np.zeros(n, SHOOT_QUERY_DTYPE)
        q["tree_a"], q["tree_b"] = tree_a, tree_b
        q["first_global"] = np.asarray(first_globals, np.float32).reshape(n, 16)
        q["second_global"] = np.asarray(second_globals, np.float32).reshape(n, 16)
        parts = []
        for i in range(n):
            ra = np.asarray(rays_first[i], np.float32).reshape(-1, 6)
            rb = np.asarray(rays_second[i], np.float32).reshape(-1, 6)
            q["n_first"][i], q["n_second"][i] = len(ra), len(rb)
            parts += [ra, rb]
        rays = np.ascontiguousarray(np.concatenate(parts) if parts else np.zeros((0, 6), np.float32))
        return q, rays

    def shoot_packed(self, queries: np.ndarray, rays: np.ndarray, params: tuple | None = None,
                     out: np.ndarray | None = None) -> np.ndarray:
        """cg_shoot_rays on a SHOOT_QUERY_DTYPE array and its (n_rays, 6) rays."""
        queries = np.ascontiguousarray(queries, SHOOT_QUERY_DTYPE)
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        n = len(queries)
        if out is None:
            out = np.zeros((max(n, 1), 3), np.float32)
        pp = None
        if params is not None:
            pp = cg_shoot_params(*[float(x) for x in params])
        self._check(self.lib.cg_shoot_rays(self.h, queries.ctypes.data if n else None, n,
                                           rays.ctypes.data if len(rays) else None, len(rays),
                                           C.byref(pp) if pp is not None else None, out.ctypes.data),
                    "cg_shoot_rays")
        return out[:n]

    def pose(self, skeleton: "Skeleton", axis_angles: int, n_poses: int, joint_matrices: int,
             stream: int | None = None):
        """cg_pose on device pointers ([n_poses][n_bones][3] -> [n_poses][n_bones][16])."""
        self._check(self.lib.cg_pose(self.h, C.byref(skeleton.view), axis_angles, n_poses, joint_matrices, stream),
                    "cg_pose")

    def pose_backward(self, skeleton: "Skeleton", axis_angles: int, joint_matrices: int, grad_joint_matrices: int,
                      n_poses: int, grad_axis_angles: int, stream: int | None = None):
        self._check(self.lib.cg_pose_backward(self.h, C.byref(skeleton.view), axis_angles, joint_matrices,
                                              grad_joint_matrices, n_poses, grad_axis_angles, stream),
                    "cg_pose_backward")

    def energy(self, d_energy: int, stream: int | None = None):
        """cg_energy into a device double."""
        self._check(self.lib.cg_energy(self.h, d_energy, stream), "cg_energy")

    def energy_backward(self, d_grad_energy: int, side_a: "EnergySide | None", side_b: "EnergySide | None" = None,
                        stream: int | None = None):
        a = C.byref(side_a.side) if side_a is not None else None
        b = C.byref(side_b.side) if side_b is not None else None
        self._check(self.lib.cg_energy_backward(self.h, d_grad_energy, a, b, stream), "cg_energy_backward")

    def device_results(self) -> tuple[int, int]:
        p, n = C.c_void_p(), C.c_void_p()
        self._check(self.lib.cg_device_results(self.h, C.byref(p), C.byref(n)), "cg_device_results")
        return p.value or 0, n.value or 0

    def traversal_ms(self) -> float:
        ms = C.c_float()
        self._check(self.lib.cg_traversal_time_ms(self.h, C.byref(ms)), "cg_traversal_time_ms")
        return ms.value

    def narrow_ms(self) -> float:
        ms = C.c_float()
        self._check(self.lib.cg_narrow_time_ms(self.h, C.byref(ms)), "cg_narrow_time_ms")
        return ms.value

    def set_trace_bucket(self, bucket_ns: int):
        self._check(self.lib.cg_read_trace(self.h, bucket_ns, None, 0), "cg_read_trace")

    def trace(self, n_buckets: int = 512) -> np.ndarray:
        """(n_buckets, 4): busy lanes, traversal steps, triangle tests, triangle passes."""
        out = np.zeros((n_buckets, 4), np.uint32)
        self._check(self.lib.cg_read_trace(self.h, 0, out.ctypes.data, n_buckets), "cg_read_trace")
        return out

    def graph_capture(self, d_queries_ptr: int, n: int, flags: int = 0):
        self._check(self.lib.cg_graph_capture(self.h, d_queries_ptr, n, flags), "cg_graph_capture")

    def graph_launch(self, stream: int | None = None):
        self._check(self.lib.cg_graph_launch(self.h, stream), "cg_graph_launch")


class Skeleton:
    """cg_skeleton_view with its host arrays kept alive: parent[j] (< j or -1)
    and offsets[j] (translation from the parent)."""

    def __init__(self, parent, offsets):
        self.parent = np.ascontiguousarray(parent, np.int32)
        self.offsets = np.ascontiguousarray(offsets, np.float32).reshape(-1, 3)
        assert len(self.parent) == len(self.offsets)
        self.view = cg_skeleton_view(len(self.parent), self.parent.ctypes.data, self.offsets.ctypes.data)

    @property
    def n_bones(self) -> int:
        return len(self.parent)


class EnergySide:
    """cg_energy_side with its view table kept alive (views: list of
    cg_deform_view, one per query; None entries are static)."""

    def __init__(self, views, joint_stride: int, target_stride: int, grad_joint_matrices: int,
                 grad_morph_weights: int | None):
        self.views = (cg_deform_view * len(views))(*[v if v is not None else cg_deform_view() for v in views])
        self.side = cg_energy_side(C.cast(self.views, C.c_void_p), joint_stride, target_stride, grad_joint_matrices,
                                   grad_morph_weights)
