"""Brute-force numpy model of the drop-in contract, for small cases.

TEST INFRASTRUCTURE ONLY (never imported by the GPU library).  It restates the
reference's per-point semantics over a flat array of points instead of a tree,
so results are independent of tree shape:

* squared distances are calc_dist (ikd-Tree/ikd_Tree.cpp:1374-1378): float32
  ((dx*dx + dy*dy) + dz*dz), each operation rounded (numpy does not fuse);
* kNN (Search, :868-1013): the k smallest distances with d2 <= max_dist^2
  compared in double (:872, :887); equal distances are ordered by point id
  (the reference leaves them to traversal order);
* Box_Search (:1015-1044): min <= p < max per axis;
* Radius_Search (:1046-1087): d2 <= r*r in float32;
* Delete_Point_Boxes (:535-556): valid points in any box become deleted;
* Delete_Points (:712-760): each input point deletes one valid point within
  EPSS = 1e-6 per axis (same_point, :1368-1371), the smallest id here;
* Add_Points with downsampling (:422-449): the voxel loop, point by point.

Point ids follow the library: Build numbers points 0..n-1; a later call with
m points reserves ids next_id .. next_id+m-1, and the point inserted for input
i gets id next_id + i.  A downsampling winner that was already in the map is
re-inserted under its own id.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


def sq_dist(q: np.ndarray, p: np.ndarray) -> np.ndarray:
    """calc_dist(q, p) broadcast, float32 unfused."""
    q = np.asarray(q, F32)
    p = np.asarray(p, F32)
    dx = q[..., 0] - p[..., 0]
    dy = q[..., 1] - p[..., 1]
    dz = q[..., 2] - p[..., 2]
    return (dx * dx + dy * dy) + dz * dz


def same_point(a, b) -> bool:
    a = np.asarray(a, F32)
    b = np.asarray(b, F32)
    return bool(np.all(np.abs(a - b).astype(np.float64) < 1e-6))


def voxel(p, ds: float):
    """Voxel box and centre of Add_Points (ikd_Tree.cpp:424-432)."""
    p = np.asarray(p, F32)
    dsf = F32(ds)
    lo = (np.floor(p / dsf) * dsf).astype(F32)
    hi = (lo + dsf).astype(F32)
    mid = (lo.astype(np.float64) + (hi - lo).astype(np.float64) / 2.0).astype(F32)
    return lo, hi, mid


class SpecTree:
    def __init__(self, downsample_size: float = 0.2):
        self.ds = downsample_size
        self.pts = np.zeros((0, 3), F32)
        self.ids = np.zeros(0, np.int64)
        self.valid = np.zeros(0, bool)
        self.next_id = 0

    # -- mutations -----------------------------------------------------------------
    def Build(self, pts):
        p = np.asarray(pts, F32).reshape(-1, 3)
        self.pts = p.copy()
        self.ids = np.arange(len(p), dtype=np.int64)
        self.valid = np.ones(len(p), bool)
        self.next_id = len(p)

    def _append(self, p, pid):
        self.pts = np.vstack([self.pts, np.asarray(p, F32).reshape(1, 3)])
        self.ids = np.append(self.ids, pid)
        self.valid = np.append(self.valid, True)

    def Add_Points(self, pts, downsample_on: bool) -> int:
        p = np.asarray(pts, F32).reshape(-1, 3)
        first = self.next_id
        self.next_id += len(p)
        if not downsample_on:
            self.pts = np.vstack([self.pts, p])
            self.ids = np.append(self.ids, first + np.arange(len(p)))
            self.valid = np.append(self.valid, np.ones(len(p), bool))
            return 0
        count = 0
        for i in range(len(p)):
            lo, hi, mid = voxel(p[i], self.ds)
            inside = np.flatnonzero(self.valid & np.all((self.pts >= lo) & (self.pts < hi), axis=1))
            inside = inside[np.argsort(self.ids[inside], kind="stable")]
            best_d = sq_dist(p[i], mid)
            winner = p[i]
            winner_id = first + i
            for j in inside:
                d = sq_dist(self.pts[j], mid)
                if d < best_d:
                    best_d = d
                    winner = self.pts[j]
                    winner_id = int(self.ids[j])
            if len(inside) > 1 or same_point(p[i], winner):
                winner = np.array(winner, F32)
                self.valid[inside] = False
                self._append(winner, winner_id)
                count += 1
        return count

    def Delete_Point_Boxes(self, boxes) -> int:
        b = np.asarray(boxes, F32).reshape(-1, 6)
        n = 0
        for bx in b:
            m = self.valid & np.all((self.pts >= bx[:3]) & (self.pts < bx[3:]), axis=1)
            n += int(m.sum())
            self.valid[m] = False
        return n

    def Delete_Points(self, pts):
        for q in np.asarray(pts, F32).reshape(-1, 3):
            close = np.all((np.abs(self.pts - q).astype(np.float64) < 1e-6), axis=1) & self.valid
            idx = np.flatnonzero(close)
            if len(idx):
                self.valid[idx[np.argmin(self.ids[idx])]] = False

    # -- searches ------------------------------------------------------------------
    def knn(self, q, k: int, max_dist: float = np.inf):
        qa = np.asarray(q, F32).reshape(-1, 3)
        vp = self.pts[self.valid]
        vid = self.ids[self.valid]
        m2 = float(max_dist) * float(max_dist)
        ids = np.full((len(qa), k), -1, np.int64)
        d2 = np.full((len(qa), k), np.inf, F32)
        for i, qq in enumerate(qa):
            d = sq_dist(qq, vp)
            ok = np.flatnonzero(d.astype(np.float64) <= m2)
            order = ok[np.lexsort((vid[ok], d[ok]))][:k]
            ids[i, :len(order)] = vid[order]
            d2[i, :len(order)] = d[order]
        return ids, d2

    def box_search(self, boxes):
        b = np.asarray(boxes, F32).reshape(-1, 6)
        return [np.sort(self.ids[self.valid & np.all((self.pts >= bx[:3]) & (self.pts < bx[3:]), axis=1)])
                for bx in b]

    def radius_search(self, q, r):
        qa = np.asarray(q, F32).reshape(-1, 3)
        ra = np.broadcast_to(np.asarray(r, F32), (len(qa),))
        out = []
        for qq, rr in zip(qa, ra):
            d = sq_dist(self.pts, qq)
            out.append(np.sort(self.ids[self.valid & (d <= F32(rr) * F32(rr))]))
        return out

    def valid_points(self):
        return self.pts[self.valid], self.ids[self.valid]

    def tree_range(self) -> np.ndarray:
        """AABB {min xyz, max xyz} of the valid points (the root's range,
        ikd_Tree.cpp:99-126); zeros for a tree without valid points."""
        v = self.valid_points()[0]
        if len(v) == 0:
            return np.zeros(6, F32)
        return np.concatenate([v.min(0), v.max(0)]).astype(F32)

    def validnum(self) -> int:
        return int(self.valid.sum())

    def size(self) -> int:
        """Stored points; the model never drops deleted ones (tree-shape dependent)."""
        return int(len(self.pts))
