"""ctypes binding for the oracle C API (oracle/oracle_capi.h).

TEST INFRASTRUCTURE ONLY.  Two interchangeable back ends expose the same API:

* ``OracleTree(kind="ref")``  - the unmodified ikd-Tree reference built by
  ``make -C oracle ref`` into ``oracle/_ref/libikd_ref.so`` (only where the
  reference sources exist);
* ``OracleTree(kind="port")`` - ``oracle/ikd_port.cpp``, the CPU restatement of
  the same algorithm, built by ``make -C oracle port``.

Only tests, ``__graft_entry__.smoke`` and ``bench.py``'s CPU-baseline leg use
this module; the GPU library never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBS = {
    "ref": os.path.join(HERE, "_ref", "libikd_ref.so"),
    "port": os.path.join(HERE, "_build", "libikd_port.so"),
}
_loaded: dict[str, C.CDLL] = {}

_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_longlong)


def build(kind: str = "port") -> str:
    """Compile the requested oracle library (make -C oracle <kind>)."""
    subprocess.run(["make", "-s", "-C", HERE, kind], check=True)
    return LIBS[kind]


def available(kind: str) -> bool:
    return os.path.exists(LIBS[kind])


def _lib(kind: str) -> C.CDLL:
    if kind in _loaded:
        return _loaded[kind]
    path = LIBS[kind]
    if not os.path.exists(path):
        raise FileNotFoundError(f"oracle library {path} is not built (make -C oracle {kind})")
    lib = C.CDLL(path)
    sig = {
        "ora_create": (C.c_void_p, [C.c_float, C.c_float, C.c_float]),
        "ora_destroy": (None, [C.c_void_p]),
        "ora_build": (None, [C.c_void_p, _fp, C.c_int]),
        "ora_add_points": (C.c_int, [C.c_void_p, _fp, C.c_int, C.c_int]),
        "ora_delete_points": (None, [C.c_void_p, _fp, C.c_int]),
        "ora_delete_boxes": (C.c_int, [C.c_void_p, _fp, C.c_int]),
        "ora_add_boxes": (None, [C.c_void_p, _fp, C.c_int]),
        "ora_knn": (None, [C.c_void_p, _fp, C.c_int, C.c_int, C.c_double, _fp, _fp, _ip, C.c_int]),
        "ora_box_search": (C.c_longlong, [C.c_void_p, _fp, C.c_int, _lp, C.c_int]),
        "ora_radius_search": (C.c_longlong, [C.c_void_p, _fp, _fp, C.c_int, _lp, C.c_int]),
        "ora_fetch": (None, [C.c_void_p, _fp]),
        "ora_flatten": (C.c_int, [C.c_void_p, _fp, C.c_int]),
        "ora_size": (C.c_int, [C.c_void_p]),
        "ora_validnum": (C.c_int, [C.c_void_p]),
        "ora_settle": (None, [C.c_void_p]),
        "ora_set_async": (None, [C.c_void_p, C.c_int]),
        "ora_acquire_removed": (C.c_int, [C.c_void_p]),
        "ora_fetch_removed": (None, [C.c_void_p, _fp]),
        "ora_tree_range": (None, [C.c_void_p, _fp]),
        "ora_root_alpha": (None, [C.c_void_p, _fp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _loaded[kind] = lib
    return lib


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def _p(a: np.ndarray):
    return a.ctypes.data_as(_fp)


class OracleTree:
    """KD_TREE<ikdTree_PointType> driven through the oracle C API."""

    def __init__(self, delete_param=0.5, balance_param=0.6, box_length=0.2, kind="port"):
        self.kind = kind
        self.lib = _lib(kind)
        self.h = self.lib.ora_create(delete_param, balance_param, box_length)

    def close(self):
        if self.h:
            self.lib.ora_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def Build(self, pts):
        a = _f32(pts).reshape(-1, 3)
        self.lib.ora_build(self.h, _p(a), a.shape[0])

    def Add_Points(self, pts, downsample_on: bool) -> int:
        a = _f32(pts).reshape(-1, 3)
        return self.lib.ora_add_points(self.h, _p(a), a.shape[0], int(bool(downsample_on)))

    def Delete_Points(self, pts):
        a = _f32(pts).reshape(-1, 3)
        self.lib.ora_delete_points(self.h, _p(a), a.shape[0])

    def Delete_Point_Boxes(self, boxes) -> int:
        b = _f32(boxes).reshape(-1, 6)
        return self.lib.ora_delete_boxes(self.h, _p(b), b.shape[0])

    def Add_Point_Boxes(self, boxes):
        b = _f32(boxes).reshape(-1, 6)
        self.lib.ora_add_boxes(self.h, _p(b), b.shape[0])

    def knn(self, q, k: int, max_dist: float = float("inf"), nthreads: int = 1):
        """Batched Nearest_Search: (xyz[nq,k,3], d2[nq,k], cnt[nq])."""
        qa = _f32(q).reshape(-1, 3)
        nq = qa.shape[0]
        xyz = np.zeros((nq, k, 3), np.float32)
        d2 = np.full((nq, k), np.inf, np.float32)
        cnt = np.zeros(nq, np.int32)
        self.lib.ora_knn(self.h, _p(qa), nq, k, float(max_dist), _p(xyz), _p(d2),
                         cnt.ctypes.data_as(_ip), nthreads)
        return xyz, d2, cnt

    def _fetch(self, counts, total):
        out = np.zeros((total, 3), np.float32)
        if total:
            self.lib.ora_fetch(self.h, _p(out))
        offs = np.zeros(len(counts) + 1, np.int64)
        np.cumsum(counts, out=offs[1:])
        return offs, out

    def box_search(self, boxes, nthreads: int = 1):
        """Batched Box_Search: (offsets[nb+1], xyz[total,3])."""
        b = _f32(boxes).reshape(-1, 6)
        counts = np.zeros(b.shape[0], np.int64)
        tot = self.lib.ora_box_search(self.h, _p(b), b.shape[0], counts.ctypes.data_as(_lp), nthreads)
        return self._fetch(counts, tot)

    def radius_search(self, q, r, nthreads: int = 1):
        qa = _f32(q).reshape(-1, 3)
        ra = _f32(np.broadcast_to(np.asarray(r, np.float32), (qa.shape[0],)))
        counts = np.zeros(qa.shape[0], np.int64)
        tot = self.lib.ora_radius_search(self.h, _p(qa), _p(ra), qa.shape[0],
                                         counts.ctypes.data_as(_lp), nthreads)
        return self._fetch(counts, tot)

    def flatten(self) -> np.ndarray:
        n = self.lib.ora_flatten(self.h, None, 0)
        out = np.zeros((n, 3), np.float32)
        if n:
            self.lib.ora_flatten(self.h, _p(out), n)
        return out

    def set_async(self, on: bool):
        """Timing mode: calls return without waiting for the reference's
        background rebuild thread (a no-op for the port)."""
        self.lib.ora_set_async(self.h, int(bool(on)))

    def settle(self):
        self.lib.ora_settle(self.h)

    def size(self) -> int:
        return self.lib.ora_size(self.h)

    def validnum(self) -> int:
        return self.lib.ora_validnum(self.h)

    def acquire_removed_points(self) -> np.ndarray:
        n = self.lib.ora_acquire_removed(self.h)
        out = np.zeros((n, 3), np.float32)
        if n:
            self.lib.ora_fetch_removed(self.h, _p(out))
        return out

    def tree_range(self) -> np.ndarray:
        out = np.zeros(6, np.float32)
        self.lib.ora_tree_range(self.h, _p(out))
        return out

    def root_alpha(self):
        out = np.zeros(2, np.float32)
        self.lib.ora_root_alpha(self.h, _p(out))
        return float(out[0]), float(out[1])
