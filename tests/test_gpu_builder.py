"""The builder's three paths at their size thresholds, on degenerate inputs.

The builder picks a path by the largest job of a call: the small CTA-local
builder (at most 1,024 points), the per-job splitter (at most 131,072 points;
radix-selected median, then the local builder) and the global sorted levels
above that (with the 4,096-point local builder at the bottom).  Each path must
give a tree that validates and answers exactly like the oracle model on
inputs whose split keys tie everywhere: every point equal, points on a plane,
points on a line with repeats, and an integer lattice with repeats.  Rebuilds
(adds of exact duplicates, then box deletions) run through the same paths.
"""
import numpy as np
import pytest

import spec

pytestmark = pytest.mark.gpu

SIZES = (1024, 1025, 4096, 4097, 131072, 131073)
KINDS = ("same", "plane", "line", "lattice")


def make(kind, n, rng):
    if kind == "same":
        return np.full((n, 3), 1.5, np.float32)
    if kind == "plane":
        p = rng.uniform(-30, 30, (n, 3)).astype(np.float32)
        p[:, 2] = 0.0
        return p
    if kind == "line":
        t = rng.integers(0, 50, n).astype(np.float32)
        return np.stack([t, 2 * t, np.zeros(n, np.float32)], 1)
    return rng.integers(-8, 8, (n, 3)).astype(np.float32)


def assert_knn(tree, ref, q, k):
    ids, d2, _, cnt = tree.knn(q, k)
    rid, rd2 = ref.knn(q, k)
    assert np.array_equal(ids, rid), f"ids differ for k={k}"
    assert np.array_equal(d2.view(np.uint32), rd2.view(np.uint32))
    assert np.array_equal(cnt, (rid >= 0).sum(1))


def assert_same_valid(tree, ref):
    xyz, ids = tree.flatten(with_ids=True)
    rxyz, rids = ref.valid_points()
    a, b = np.argsort(ids, kind="stable"), np.argsort(rids, kind="stable")
    assert np.array_equal(np.asarray(ids)[a], np.asarray(rids)[b])
    assert np.array_equal(np.asarray(xyz, np.float32)[a].view(np.uint32),
                          np.asarray(rxyz, np.float32)[b].view(np.uint32))
    assert tree.validnum() == ref.validnum()


def queries(pts, rng, m=150):
    q = pts[rng.choice(len(pts), m)] + rng.normal(0, 0.7, (m, 3)).astype(np.float32)
    return np.concatenate([q, pts[rng.choice(len(pts), 30)]]).astype(np.float32)


def boxes_around(pts, rng, m=6):
    c = pts[rng.choice(len(pts), m)]
    h = rng.uniform(0.5, 4.0, (m, 3)).astype(np.float32)
    return np.concatenate([c - h, c + h], 1).astype(np.float32)


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("kind", KINDS)
def test_build_paths_degenerate(ikdg_mod, kind, n):
    rng = np.random.default_rng(n * 11 + KINDS.index(kind))
    pts = make(kind, n, rng)
    tree, ref = ikdg_mod.KDTree(), spec.SpecTree()
    tree.Build(pts)
    ref.Build(pts)
    assert tree.validate() == 0
    assert tree.validnum() == n
    q = queries(pts, rng, 150 if n < 100000 else 40)  # the model's brute force is the slow side
    for k in (1, 5, 16):
        assert_knn(tree, ref, q, k)
    bx = boxes_around(pts, rng)
    offs, ids, _ = tree.box_search(bx)
    for i, want in enumerate(ref.box_search(bx)):
        assert np.array_equal(np.sort(ids[offs[i]:offs[i + 1]]), want)
    tree.close()


@pytest.mark.parametrize("kind", ("plane", "lattice"))
def test_rebuilds_on_duplicates(ikdg_mod, kind):
    rng = np.random.default_rng(77 + KINDS.index(kind))
    pts = make(kind, 20000, rng)
    tree, ref = ikdg_mod.KDTree(), spec.SpecTree()
    tree.Build(pts)
    ref.Build(pts)
    # Exact duplicates of existing points in growing batches unbalance the
    # subtrees they land in; the rebuilds split on tied keys.
    for step in range(4):
        add = pts[rng.choice(len(pts), 3000 * (step + 1))].copy()
        assert tree.Add_Points(add, False) == ref.Add_Points(add, False)
        assert tree.validate() == 0
    bx = boxes_around(pts, rng, 12)
    assert tree.Delete_Point_Boxes(bx) == ref.Delete_Point_Boxes(bx)
    assert tree.validate() == 0
    assert_same_valid(tree, ref)
    q = queries(pts, rng)
    for k in (1, 8, 16):
        assert_knn(tree, ref, q, k)
    tree.close()


def test_two_large_rebuild_jobs(ikdg_mod):
    # A 4 x 1 x 1 slab: the root and its children split x at the quartiles.
    # Deleting 60 % of the first and of the last quarter makes those two
    # subtrees (400k points each) violate the delete criterion while the
    # halves and the root stay within it: the call aims at two rebuild jobs
    # of ~160k valid points each, the global sorted path with two jobs.
    rng = np.random.default_rng(4242)
    n = 1_600_000
    pts = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    pts[:, 0] *= 4
    tree, ref = ikdg_mod.KDTree(), spec.SpecTree()
    tree.Build(pts)
    ref.Build(pts)
    bx = np.array([[-1, -1, -1, 0.6, 2, 2], [3.4, -1, -1, 5, 2, 2]], np.float32)
    assert tree.Delete_Point_Boxes(bx) == ref.Delete_Point_Boxes(bx)
    assert tree.validate() == 0
    assert tree.validnum() == ref.validnum()
    q = rng.uniform([-0.2, -0.1, -0.1], [4.2, 1.1, 1.1], (30, 3)).astype(np.float32)
    for k in (1, 8):
        assert_knn(tree, ref, q, k)
    xyz, ids = tree.flatten(with_ids=True)
    assert np.array_equal(np.sort(ids), np.sort(ref.valid_points()[1]))
    tree.close()
