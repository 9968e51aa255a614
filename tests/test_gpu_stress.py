"""Scale stress at full size: a 20M-point map, 1M-query batches.

The map is uniform in [-500, 500]^2 x [0, 50] m plus planar clusters; 1M
uniform queries run kNN at k in {1, 5, 16, 32} with max_dist = 2 m and a
radius search with r = 1 m; then 1000 boxes (sides 1-20 m) are deleted (the
deletions trigger rebuilds) and the same queries run again.  An oracle at this
size is too slow, so the checks are size-independent properties plus exact
answers for a sample of queries:

* every row is sorted by (squared distance, id), within max_dist, and its
  squared distances recompute bit for bit from the returned points;
* the k-row is exactly the first k entries of the 32-row (prefix property);
* radius hits equal the 32-row entries within r wherever the 32-row is not
  full, and contain them everywhere;
* 2000 sampled queries match an exact brute force over candidates gathered
  by scipy's cKDTree (squared distances recomputed in float32 with the
  reference's formula, ties by id);
* the number deleted equals the number of valid points in the union of the
  boxes (numpy), validnum drops by it, no deleted id is ever returned again,
  and the device structure validates.
"""
import math

import numpy as np
import pytest

import synthetic as S

pytestmark = pytest.mark.gpu

N = 20_000_000
NQ = 1_000_000
KS = (1, 5, 16, 32)
MAX_DIST = 2.0
R = 1.0
F32 = np.float32


def sq(q, p):
    dx, dy, dz = q[..., 0] - p[..., 0], q[..., 1] - p[..., 1], q[..., 2] - p[..., 2]
    return (dx * dx + dy * dy) + dz * dz


def thr(d):
    """Largest float32 <= d*d (d*d in double): the acceptance bound."""
    t = np.float32(d * d)
    return t if float(t) <= d * d else np.nextafter(t, F32(0))


def check_rows(q, ids, d2, xyz, cnt, k, bound):
    n = len(q)
    col = np.arange(k)[None, :]
    valid = col < cnt[:, None]
    assert np.all(cnt <= k) and np.all(cnt >= 0)
    assert np.all(ids[~valid] == -1)
    assert np.all(d2[valid] <= bound)
    # sorted by (d2, id)
    a, b = d2[:, :-1], d2[:, 1:]
    both = valid[:, 1:]
    assert np.all((a < b) | ((a == b) & (ids[:, :-1] < ids[:, 1:])) | ~both)
    # distances recompute exactly from the points
    rec = sq(q[:, None, :], xyz)
    assert np.array_equal(rec[valid].view(np.uint32), d2[valid].view(np.uint32))


def brute(ckd, pts, live_ids, q, k, bound):
    """Exact (d2, id) top-k of float32 squared distances among live points."""
    cand = ckd.query_ball_point(q.astype(np.float64), math.sqrt(float(bound)) + 1e-3)
    out_ids = np.full((len(q), k), -1, np.int64)
    out_d2 = np.full((len(q), k), np.inf, F32)
    for i, c in enumerate(cand):
        c = np.asarray(c, np.int64)
        gid = live_ids[c]
        d = sq(q[i], pts[gid])
        ok = d <= bound
        gid, d = gid[ok], d[ok]
        o = np.lexsort((gid, d))[:k]
        out_ids[i, :len(o)] = gid[o]
        out_d2[i, :len(o)] = d[o]
    return out_ids, out_d2


def deleted_mask(pts, boxes):
    order = np.argsort(pts[:, 0], kind="stable")
    xs = pts[order, 0]
    mask = np.zeros(len(pts), bool)
    for b in boxes:
        lo, hi = np.searchsorted(xs, b[0], "left"), np.searchsorted(xs, b[3], "left")
        idx = order[lo:hi]
        p = pts[idx]
        inb = np.all((p >= b[:3]) & (p < b[3:]), axis=1)
        mask[idx[inb]] = True
    return mask


@pytest.fixture(scope="module")
def world(ikdg_mod):
    pts = S.stress_map(N, 5005)
    rng = np.random.default_rng(5006)
    q = np.empty((NQ, 3), F32)
    q[:, :2] = rng.uniform(-500, 500, (NQ, 2))
    q[:, 2] = rng.uniform(0, 50, NQ)
    tree = ikdg_mod.KDTree(0.5, 0.6, 0.5)
    tree.Build(pts)
    yield pts, q, tree
    tree.close()


def run_queries(tree, q):
    bound = thr(MAX_DIST)
    res = {}
    for k in KS:
        ids, d2, xyz, cnt = tree.knn(q, k, MAX_DIST)
        check_rows(q, ids, d2, xyz, cnt, k, bound)
        res[k] = (ids, d2, cnt)
    i32, d32, c32 = res[32]
    for k in KS[:-1]:
        ids, d2, cnt = res[k]
        assert np.array_equal(cnt, np.minimum(c32, k)), f"k={k}: counts"
        assert np.array_equal(ids, i32[:, :k]), f"k={k}: not a prefix of k=32"
        assert np.array_equal(d2.view(np.uint32), d32[:, :k].view(np.uint32))
    offs, rids, rxyz = tree.radius_search(q, R)
    rc = np.diff(offs)
    r2 = F32(R) * F32(R)
    within = (d32 <= r2) & (np.arange(32)[None, :] < c32[:, None])
    nw = within.sum(1)
    assert np.all(nw <= rc)
    full = c32 == 32
    assert np.array_equal(nw[~full], rc[~full]), "radius hits differ from kNN within r"
    sample = np.flatnonzero(~full)[:50000]
    for i in sample[rc[sample] > 0][:5000]:
        got = np.sort(rids[offs[i]:offs[i + 1]])
        assert np.array_equal(got, np.sort(i32[i][within[i]])), f"query {i}: radius set"
    return res


def test_stress_queries_and_deletes(world):
    spatial = pytest.importorskip("scipy.spatial")
    pts, q, tree = world
    assert tree.validnum() == N
    res = run_queries(tree, q)
    bound = thr(MAX_DIST)
    live = np.arange(N)
    ckd = spatial.cKDTree(pts.astype(np.float64))
    rng = np.random.default_rng(9)
    sample = rng.choice(NQ, 2000, replace=False)
    bi, bd = brute(ckd, pts, live, q[sample], 32, bound)
    i32, d32, c32 = res[32]
    assert np.array_equal(i32[sample], bi) and np.array_equal(d32[sample].view(np.uint32), bd.view(np.uint32))

    boxes = S.random_boxes(1000, 5007)
    mask = deleted_mask(pts, boxes)
    n_del = tree.Delete_Point_Boxes(boxes)
    assert n_del == int(mask.sum())
    assert tree.validnum() == N - n_del
    assert tree.validate() == 0

    res2 = run_queries(tree, q)
    for k in KS:
        ids = res2[k][0]
        got = ids[ids >= 0]
        assert not mask[got].any(), f"k={k}: a deleted point was returned"
    live = np.flatnonzero(~mask)
    ckd2 = spatial.cKDTree(pts[live].astype(np.float64))
    bi, bd = brute(ckd2, pts, live, q[sample], 32, bound)
    i32, d32, c32 = res2[32]
    assert np.array_equal(i32[sample], bi) and np.array_equal(d32[sample].view(np.uint32), bd.view(np.uint32))
