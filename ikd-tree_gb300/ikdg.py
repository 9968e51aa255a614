"""Python binding of libikdg (the GB300 incremental k-d tree) over its C ABI.

``KDTree`` mirrors ``KD_TREE<PointType>`` (ikd-Tree/ikd_Tree.h:225-248): same
method names, argument meaning and return values, plus batched forms of the
searches (``knn``, ``box_search``, ``radius_search``) that take all queries of a
step at once.  Every method runs CUDA kernels through libikdg.so; there is no
CPU code path, and constructing a tree without the library or without a GPU
raises.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libikdg.so")

OK, BAD_ARG, CAPACITY, DEVICE_TIMEOUT, CUDA_ERR, NO_DEVICE, INTERNAL = 0, 2, 3, 4, 5, 6, 7

_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)
_vp = C.c_void_p

# Every entry point of include/ikdg.h with its ctypes signature.
SIGNATURES = {
    "ikdg_status_string": (C.c_char_p, [C.c_int]),
    "ikdg_last_error": (C.c_char_p, [_vp]),
    "ikdg_create": (C.c_int, [C.c_float, C.c_float, C.c_float, C.c_int, C.POINTER(_vp)]),
    "ikdg_destroy": (C.c_int, [_vp]),
    "ikdg_set_delete_criterion_param": (C.c_int, [_vp, C.c_float]),
    "ikdg_set_balance_criterion_param": (C.c_int, [_vp, C.c_float]),
    "ikdg_set_downsample_param": (C.c_int, [_vp, C.c_float]),
    "ikdg_set_leaf_fill": (C.c_int, [_vp, C.c_int]),
    "ikdg_set_knn_lanes": (C.c_int, [_vp, C.c_int]),
    "ikdg_set_knn_bin_bits": (C.c_int, [_vp, C.c_int]),
    "ikdg_build": (C.c_int, [_vp, _fp, C.c_int64, C.c_int32]),
    "ikdg_add_points": (C.c_int, [_vp, _fp, C.c_int64, C.c_int32, C.c_int, _lp]),
    "ikdg_delete_points": (C.c_int, [_vp, _fp, C.c_int64, C.c_int32]),
    "ikdg_delete_boxes": (C.c_int, [_vp, _fp, C.c_int64, _lp]),
    "ikdg_add_boxes": (C.c_int, [_vp, _fp, C.c_int64]),
    "ikdg_knn": (C.c_int, [_vp, _fp, C.c_int64, C.c_int32, C.c_int32, C.c_double, _ip, _fp, _fp, _ip]),
    "ikdg_knn_device": (C.c_int, [_vp, _vp, C.c_int64, C.c_int32, C.c_int32, C.c_double, _vp, _vp, _vp, _vp]),
    "ikdg_knn_device_noalloc": (C.c_int, [_vp, _vp, C.c_int64, C.c_int32, C.c_int32, C.c_double, _vp, _vp, _vp,
                                          _vp]),
    "ikdg_box_search": (C.c_int, [_vp, _fp, C.c_int64, _lp, _ip, _fp, C.c_int64, _lp]),
    "ikdg_radius_search": (C.c_int, [_vp, _fp, C.c_int64, C.c_int32, _fp, C.c_int32, _lp, _ip, _fp, C.c_int64,
                                     _lp]),
    "ikdg_p2p_forward": (C.c_int, [_vp, _vp, C.c_int64, C.POINTER(C.c_double), C.c_int32, C.c_double, C.c_float,
                                   _vp, _vp, _vp, C.POINTER(C.c_double)]),
    "ikdg_p2p_adjoint": (C.c_int, [_vp, _vp, C.c_int64, C.POINTER(C.c_double), _vp, _vp, _vp, C.c_double, _vp,
                                   C.POINTER(C.c_double)]),
    "ikdg_size": (C.c_int, [_vp, _lp]),
    "ikdg_validnum": (C.c_int, [_vp, _lp]),
    "ikdg_tree_range": (C.c_int, [_vp, _fp]),
    "ikdg_root_alpha": (C.c_int, [_vp, _fp, _fp]),
    "ikdg_flatten": (C.c_int, [_vp, _fp, _ip, C.c_int64, _lp]),
    "ikdg_acquire_removed_points": (C.c_int, [_vp, _fp, _ip, C.c_int64, _lp]),
    "ikdg_live_ids": (C.c_int, [_vp, _ip, C.c_int64, _lp]),
    "ikdg_rebuild": (C.c_int, [_vp]),
    "ikdg_debug_validate": (C.c_int, [_vp, _lp]),
    "ikdg_get_stream": (C.c_int, [_vp, C.POINTER(_vp)]),
    "ikdg_set_stream": (C.c_int, [_vp, _vp]),
    "ikdg_synchronize": (C.c_int, [_vp]),
    "ikdg_box_search_device": (C.c_int, [_vp, _vp, C.c_int64, _vp, _vp, _vp, C.c_int64, _vp]),
    "ikdg_radius_search_device": (C.c_int, [_vp, _vp, C.c_int64, C.c_int32, _vp, C.c_int32, _vp, _vp, _vp,
                                            C.c_int64, _vp]),
    "ikdg_batch_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "ikdg_batch_destroy": (C.c_int, [_vp]),
    "ikdg_batch_clear": (C.c_int, [_vp]),
    "ikdg_batch_last_error": (C.c_char_p, [_vp]),
    "ikdg_batch_add_knn": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int32, C.c_int32, C.c_double, _vp, _vp, _vp,
                                     _vp, _ip]),
    "ikdg_batch_add_box_search": (C.c_int, [_vp, _vp, _vp, C.c_int64, _vp, _vp, _vp, C.c_int64, _ip]),
    "ikdg_batch_add_radius_search": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int32, _vp, C.c_int32, _vp, _vp,
                                               _vp, C.c_int64, _ip]),
    "ikdg_batch_set_knn_lanes": (C.c_int, [_vp, C.c_int32, C.c_int32]),
    "ikdg_batch_set_graph": (C.c_int, [_vp, C.c_int]),
    "ikdg_batch_set_query_order": (C.c_int, [_vp, C.c_int]),
    "ikdg_batch_run": (C.c_int, [_vp]),
    "ikdg_batch_synchronize": (C.c_int, [_vp, _lp]),
    "ikdg_batch_autotune": (C.c_int, [_vp, C.c_int32, _ip]),
    "ikdg_batch_num_trees": (C.c_int, [_vp, _ip]),
    "ikdg_batch_get_stream": (C.c_int, [_vp, C.POINTER(_vp)]),
}

_lib = None


class IkdgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"ikdg error {status}: {msg}")
        self.status = status


def load(path: str = LIB_PATH) -> C.CDLL:
    """Loads libikdg.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} is missing: build it with `python ikd-tree_gb300/build.py` (the GPU path has no fallback)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _f32(a, width: int) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    return a.reshape(-1, width)


def _p(a):
    return None if a is None else a.ctypes.data_as(_fp)


class KDTree:
    """KD_TREE<PointType> on the GPU (xyz points, float32)."""

    def __init__(self, delete_param: float = 0.5, balance_param: float = 0.6, box_length: float = 0.2,
                 device: int = -1):
        self.lib = load()
        h = _vp()
        st = self.lib.ikdg_create(delete_param, balance_param, box_length, device, C.byref(h))
        if st != OK:
            raise IkdgError(st, self.lib.ikdg_status_string(st).decode())
        self.h = h

    # -- plumbing --------------------------------------------------------------
    def _check(self, st: int, what: str):
        if st != OK:
            msg = self.lib.ikdg_last_error(self.h).decode() if self.h else ""
            raise IkdgError(st, f"{what}: {self.lib.ikdg_status_string(st).decode()} ({msg})")

    def close(self):
        if getattr(self, "h", None):
            self.lib.ikdg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- parameters (ikd_Tree.h:228-231) -----------------------------------------
    def Set_delete_criterion_param(self, v: float):
        self._check(self.lib.ikdg_set_delete_criterion_param(self.h, v), "Set_delete_criterion_param")

    def Set_balance_criterion_param(self, v: float):
        self._check(self.lib.ikdg_set_balance_criterion_param(self.h, v), "Set_balance_criterion_param")

    def set_downsample_param(self, v: float):
        self._check(self.lib.ikdg_set_downsample_param(self.h, v), "set_downsample_param")

    def InitializeKDTree(self, delete_param=0.5, balance_param=0.7, box_length=0.2):
        self.Set_delete_criterion_param(delete_param)
        self.Set_balance_criterion_param(balance_param)
        self.set_downsample_param(box_length)

    def set_leaf_fill(self, fill: int):
        self._check(self.lib.ikdg_set_leaf_fill(self.h, fill), "set_leaf_fill")

    def set_knn_lanes(self, lanes: int):
        self._check(self.lib.ikdg_set_knn_lanes(self.h, lanes), "set_knn_lanes")

    def set_knn_bin_bits(self, bits: int):
        self._check(self.lib.ikdg_set_knn_bin_bits(self.h, bits), "set_knn_bin_bits")

    # -- mutations -------------------------------------------------------------
    def Build(self, pts):
        a = _f32(pts, 3)
        self._check(self.lib.ikdg_build(self.h, _p(a), a.shape[0], 3), "Build")

    def Add_Points(self, pts, downsample_on: bool) -> int:
        a = _f32(pts, 3)
        n = C.c_int64(0)
        self._check(self.lib.ikdg_add_points(self.h, _p(a), a.shape[0], 3, int(bool(downsample_on)), C.byref(n)),
                    "Add_Points")
        return n.value

    def Delete_Points(self, pts):
        a = _f32(pts, 3)
        self._check(self.lib.ikdg_delete_points(self.h, _p(a), a.shape[0], 3), "Delete_Points")

    def Delete_Point_Boxes(self, boxes) -> int:
        b = _f32(boxes, 6)
        n = C.c_int64(0)
        self._check(self.lib.ikdg_delete_boxes(self.h, _p(b), b.shape[0], C.byref(n)), "Delete_Point_Boxes")
        return n.value

    def Add_Point_Boxes(self, boxes):
        b = _f32(boxes, 6)
        self._check(self.lib.ikdg_add_boxes(self.h, _p(b), b.shape[0]), "Add_Point_Boxes")

    def rebuild(self):
        self._check(self.lib.ikdg_rebuild(self.h), "rebuild")

    # -- searches --------------------------------------------------------------
    def knn(self, q, k: int, max_dist: float = math.inf, want_xyz: bool = True):
        """Batched Nearest_Search: (ids[nq,k], d2[nq,k], xyz[nq,k,3] or None, count[nq])."""
        qa = _f32(q, 3)
        nq = qa.shape[0]
        ids = np.empty((nq, k), np.int32)
        d2 = np.empty((nq, k), np.float32)
        xyz = np.empty((nq, k, 3), np.float32) if want_xyz else None
        cnt = np.empty(nq, np.int32)
        self._check(self.lib.ikdg_knn(self.h, _p(qa), nq, 3, k, float(max_dist), ids.ctypes.data_as(_ip), _p(d2),
                                      _p(xyz), cnt.ctypes.data_as(_ip)), "knn")
        return ids, d2, xyz, cnt

    def knn_into(self, q_ptr: int, nq: int, k: int, max_dist: float, ids_ptr: int, d2_ptr: int, xyz_ptr: int = 0,
                 cnt_ptr: int = 0, stride: int = 3):
        """ikdg_knn on caller-owned HOST buffers given as raw addresses (synchronous)."""
        self._check(self.lib.ikdg_knn(self.h, C.cast(q_ptr, _fp), nq, stride, k, float(max_dist),
                                      C.cast(ids_ptr, _ip), C.cast(d2_ptr, _fp),
                                      C.cast(xyz_ptr, _fp) if xyz_ptr else None,
                                      C.cast(cnt_ptr, _ip) if cnt_ptr else None), "knn")

    def Nearest_Search(self, point, k: int, max_dist: float = math.inf):
        """Single query, reference signature: returns (points[c,3], distances[c])."""
        ids, d2, xyz, cnt = self.knn(np.asarray(point, np.float32).reshape(1, 3), k, max_dist)
        c = int(cnt[0])
        return xyz[0, :c].copy(), d2[0, :c].copy()

    def _range(self, fn, args, nq):
        offs = np.zeros(nq + 1, np.int64)
        total = C.c_int64(0)
        st = fn(*args(offs, None, None, 0, total))
        if st not in (OK, CAPACITY):
            self._check(st, "range search")
        t = total.value
        ids = np.empty(max(t, 1), np.int32)
        xyz = np.empty((max(t, 1), 3), np.float32)
        if t > 0:
            self._check(fn(*args(offs, ids, xyz, t, total)), "range search")
        return offs, ids[:t], xyz[:t]

    def box_search(self, boxes):
        """Batched Box_Search: (offsets[nb+1], ids[total], xyz[total,3])."""
        b = _f32(boxes, 6)
        nb = b.shape[0]

        def args(offs, ids, xyz, cap, total):
            return (self.h, _p(b), nb, offs.ctypes.data_as(_lp),
                    None if ids is None else ids.ctypes.data_as(_ip), _p(xyz), cap, C.byref(total))
        return self._range(self.lib.ikdg_box_search, args, nb)

    def radius_search(self, q, radius):
        """Batched Radius_Search: (offsets[nq+1], ids[total], xyz[total,3])."""
        qa = _f32(q, 3)
        nq = qa.shape[0]
        r = np.ascontiguousarray(np.broadcast_to(np.asarray(radius, np.float32), (nq,)))

        def args(offs, ids, xyz, cap, total):
            return (self.h, _p(qa), nq, 3, _p(r), 1, offs.ctypes.data_as(_lp),
                    None if ids is None else ids.ctypes.data_as(_ip), _p(xyz), cap, C.byref(total))
        return self._range(self.lib.ikdg_radius_search, args, nq)

    def Box_Search(self, box):
        offs, ids, xyz = self.box_search(np.asarray(box, np.float32).reshape(1, 6))
        return xyz

    def Radius_Search(self, point, radius: float):
        offs, ids, xyz = self.radius_search(np.asarray(point, np.float32).reshape(1, 3), radius)
        return xyz

    # -- state -------------------------------------------------------------------
    def size(self) -> int:
        n = C.c_int64(0)
        self._check(self.lib.ikdg_size(self.h, C.byref(n)), "size")
        return n.value

    def validnum(self) -> int:
        n = C.c_int64(0)
        self._check(self.lib.ikdg_validnum(self.h, C.byref(n)), "validnum")
        return n.value

    def tree_range(self) -> np.ndarray:
        out = np.zeros(6, np.float32)
        self._check(self.lib.ikdg_tree_range(self.h, _p(out)), "tree_range")
        return out

    def root_alpha(self):
        b = C.c_float(0)
        d = C.c_float(0)
        self._check(self.lib.ikdg_root_alpha(self.h, C.byref(b), C.byref(d)), "root_alpha")
        return b.value, d.value

    def flatten(self, with_ids: bool = False):
        n = C.c_int64(0)
        st = self.lib.ikdg_flatten(self.h, None, None, 0, C.byref(n))
        if st not in (OK, CAPACITY):
            self._check(st, "flatten")
        k = n.value
        xyz = np.empty((max(k, 1), 3), np.float32)
        ids = np.empty(max(k, 1), np.int32)
        if k > 0:
            self._check(self.lib.ikdg_flatten(self.h, _p(xyz), ids.ctypes.data_as(_ip), k, C.byref(n)), "flatten")
        return (xyz[:k], ids[:k]) if with_ids else xyz[:k]

    def acquire_removed_points(self, with_ids: bool = False):
        n = C.c_int64(0)
        st = self.lib.ikdg_acquire_removed_points(self.h, None, None, 0, C.byref(n))
        if st == OK and n.value == 0:
            empty = np.zeros((0, 3), np.float32)
            return (empty, np.zeros(0, np.int32)) if with_ids else empty
        if st not in (OK, CAPACITY):
            self._check(st, "acquire_removed_points")
        k = n.value
        xyz = np.empty((k, 3), np.float32)
        ids = np.empty(k, np.int32)
        self._check(self.lib.ikdg_acquire_removed_points(self.h, _p(xyz), ids.ctypes.data_as(_ip), k, C.byref(n)),
                    "acquire_removed_points")
        return (xyz, ids) if with_ids else xyz

    def live_ids(self) -> np.ndarray:
        """Ids the tree can still return: stored (valid or deleted) points and
        removed points not yet acquired."""
        n = C.c_int64(0)
        st = self.lib.ikdg_live_ids(self.h, None, 0, C.byref(n))
        if st not in (OK, CAPACITY):
            self._check(st, "live_ids")
        k = n.value
        ids = np.empty(max(k, 1), np.int32)
        if k > 0:
            self._check(self.lib.ikdg_live_ids(self.h, ids.ctypes.data_as(_ip), k, C.byref(n)), "live_ids")
        return ids[:k]

    def validate(self) -> int:
        """Structural violations of the device tree (0 = sound)."""
        n = C.c_int64(0)
        self._check(self.lib.ikdg_debug_validate(self.h, C.byref(n)), "debug_validate")
        return n.value

    # -- streams ---------------------------------------------------------------
    def stream(self) -> int:
        """The tree's CUDA stream (destroyed with the tree: free torch tensors
        whose work ran on it, e.g. under torch.cuda.ExternalStream, first)."""
        s = _vp()
        self._check(self.lib.ikdg_get_stream(self.h, C.byref(s)), "get_stream")
        return s.value or 0

    def synchronize(self):
        self._check(self.lib.ikdg_synchronize(self.h), "synchronize")

    def p2p_forward(self, scan_ptr: int, n: int, pose, k: int, max_dist: float, plane_thresh: float,
                    planes_ptr: int, res_ptr: int, valid_ptr: int) -> float:
        """Point-to-plane residuals on device buffers; returns the loss."""
        pz = (C.c_double * 6)(*[float(v) for v in pose])
        loss = C.c_double(0)
        self._check(self.lib.ikdg_p2p_forward(self.h, _vp(scan_ptr), n, pz, k, float(max_dist), float(plane_thresh),
                                              _vp(planes_ptr), _vp(res_ptr), _vp(valid_ptr), C.byref(loss)),
                    "p2p_forward")
        return loss.value

    def p2p_adjoint(self, scan_ptr: int, n: int, pose, planes_ptr: int, res_ptr: int, valid_ptr: int,
                    grad_loss: float, grad_points_ptr: int = 0):
        """Adjoint of p2p_forward; returns dL/d(omega, t) (6 floats)."""
        pz = (C.c_double * 6)(*[float(v) for v in pose])
        g = (C.c_double * 6)()
        self._check(self.lib.ikdg_p2p_adjoint(self.h, _vp(scan_ptr), n, pz, _vp(planes_ptr), _vp(res_ptr),
                                              _vp(valid_ptr), float(grad_loss), _vp(grad_points_ptr or None), g),
                    "p2p_adjoint")
        return list(g)

    def knn_device_noalloc(self, q_ptr: int, nq: int, k: int, max_dist: float, ids_ptr: int, d2_ptr: int,
                           xyz_ptr: int = 0, cnt_ptr: int = 0, stride: int = 3):
        """kNN on device buffers that allocates no device memory (see ikdg.h)."""
        self._check(self.lib.ikdg_knn_device_noalloc(self.h, _vp(q_ptr), nq, stride, k, float(max_dist),
                                                     _vp(ids_ptr), _vp(d2_ptr), _vp(xyz_ptr or None),
                                                     _vp(cnt_ptr or None)), "knn_device_noalloc")

    def knn_device(self, q_ptr: int, nq: int, k: int, max_dist: float, ids_ptr: int, d2_ptr: int,
                   xyz_ptr: int = 0, cnt_ptr: int = 0, stride: int = 3):
        """kNN on device buffers (raw pointers), asynchronous on the tree's stream."""
        self._check(self.lib.ikdg_knn_device(self.h, _vp(q_ptr), nq, stride, k, float(max_dist), _vp(ids_ptr),
                                             _vp(d2_ptr), _vp(xyz_ptr or None), _vp(cnt_ptr or None)),
                    "knn_device")

    def box_search_device(self, boxes_ptr: int, nb: int, offsets_ptr: int, ids_ptr: int, capacity: int,
                          xyz_ptr: int = 0, total_ptr: int = 0):
        """Box_Search over device buffers (CSR), asynchronous on the tree's stream."""
        self._check(self.lib.ikdg_box_search_device(self.h, _vp(boxes_ptr or None), nb, _vp(offsets_ptr),
                                                    _vp(ids_ptr or None), _vp(xyz_ptr or None), capacity,
                                                    _vp(total_ptr or None)), "box_search_device")

    def radius_search_device(self, centers_ptr: int, nq: int, radius_ptr: int, offsets_ptr: int, ids_ptr: int,
                             capacity: int, xyz_ptr: int = 0, total_ptr: int = 0, stride: int = 3,
                             radius_stride: int = 1):
        """Radius_Search over device buffers (CSR), asynchronous on the tree's stream."""
        self._check(self.lib.ikdg_radius_search_device(self.h, _vp(centers_ptr or None), nq, stride,
                                                       _vp(radius_ptr or None), radius_stride, _vp(offsets_ptr),
                                                       _vp(ids_ptr or None), _vp(xyz_ptr or None), capacity,
                                                       _vp(total_ptr or None)), "radius_search_device")


class Batch:
    """Many searches over many trees, run as one CUDA graph (see ikdg.h).

    Requests take device pointers (e.g. ``tensor.data_ptr()``) that must stay
    valid while the batch holds them."""

    def __init__(self, device: int = -1):
        self.lib = load()
        h = _vp()
        st = self.lib.ikdg_batch_create(device, C.byref(h))
        if st != OK:
            raise IkdgError(st, self.lib.ikdg_status_string(st).decode())
        self.h = h
        self._keep = []  # trees referenced by requests

    def _check(self, st: int, what: str):
        if st != OK:
            msg = self.lib.ikdg_batch_last_error(self.h).decode() if self.h else ""
            raise IkdgError(st, f"{what}: {self.lib.ikdg_status_string(st).decode()} ({msg})")

    def close(self):
        if getattr(self, "h", None):
            self.lib.ikdg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clear(self):
        self._check(self.lib.ikdg_batch_clear(self.h), "batch_clear")
        self._keep = []

    def add_knn(self, tree: KDTree, q_ptr: int, nq: int, k: int, max_dist: float, ids_ptr: int, d2_ptr: int,
                xyz_ptr: int = 0, cnt_ptr: int = 0, stride: int = 3) -> int:
        r = C.c_int32()
        self._check(self.lib.ikdg_batch_add_knn(self.h, tree.h, _vp(q_ptr or None), nq, stride, k, float(max_dist),
                                                _vp(ids_ptr or None), _vp(d2_ptr or None), _vp(xyz_ptr or None),
                                                _vp(cnt_ptr or None), C.byref(r)), "batch_add_knn")
        self._keep.append(tree)
        return r.value

    def add_box_search(self, tree: KDTree, boxes_ptr: int, nb: int, offsets_ptr: int, ids_ptr: int, capacity: int,
                       xyz_ptr: int = 0) -> int:
        r = C.c_int32()
        self._check(self.lib.ikdg_batch_add_box_search(self.h, tree.h, _vp(boxes_ptr or None), nb, _vp(offsets_ptr),
                                                       _vp(ids_ptr or None), _vp(xyz_ptr or None), capacity,
                                                       C.byref(r)), "batch_add_box_search")
        self._keep.append(tree)
        return r.value

    def add_radius_search(self, tree: KDTree, centers_ptr: int, nq: int, radius_ptr: int, offsets_ptr: int,
                          ids_ptr: int, capacity: int, xyz_ptr: int = 0, stride: int = 3,
                          radius_stride: int = 1) -> int:
        r = C.c_int32()
        self._check(self.lib.ikdg_batch_add_radius_search(self.h, tree.h, _vp(centers_ptr or None), nq, stride,
                                                          _vp(radius_ptr or None), radius_stride, _vp(offsets_ptr),
                                                          _vp(ids_ptr or None), _vp(xyz_ptr or None), capacity,
                                                          C.byref(r)), "batch_add_radius_search")
        self._keep.append(tree)
        return r.value

    def set_knn_lanes(self, request: int, lanes: int):
        self._check(self.lib.ikdg_batch_set_knn_lanes(self.h, request, lanes), "batch_set_knn_lanes")

    def set_graph(self, use_graph: bool):
        self._check(self.lib.ikdg_batch_set_graph(self.h, 1 if use_graph else 0), "batch_set_graph")

    def set_query_order(self, ordered: bool):
        """Search every request's queries in spatial (Morton) order (default on)."""
        self._check(self.lib.ikdg_batch_set_query_order(self.h, 1 if ordered else 0), "batch_set_query_order")

    def run(self):
        self._check(self.lib.ikdg_batch_run(self.h), "batch_run")

    def synchronize(self, n_range: int = 0) -> np.ndarray:
        """Waits for the last run; returns the totals of the range requests."""
        tot = np.zeros(max(n_range, 1), np.int64)
        self._check(self.lib.ikdg_batch_synchronize(self.h, tot.ctypes.data_as(_lp)), "batch_synchronize")
        return tot[:n_range]

    def autotune(self, reps: int = 3) -> np.ndarray:
        """Picks leaf fill and kNN lanes per tree; returns {fill, lanes} rows."""
        n = C.c_int32()
        self._check(self.lib.ikdg_batch_num_trees(self.h, C.byref(n)), "batch_num_trees")
        out = np.zeros((max(n.value, 1), 2), np.int32)
        self._check(self.lib.ikdg_batch_autotune(self.h, reps, out.ctypes.data_as(_ip)), "batch_autotune")
        return out[:n.value]

    @property
    def stream(self) -> int:
        s = _vp()
        self._check(self.lib.ikdg_batch_get_stream(self.h, C.byref(s)), "batch_get_stream")
        return s.value or 0
