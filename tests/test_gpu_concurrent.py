"""Concurrent Nearest_Search callers (ikd_Tree.cpp:875-884: the reference lets
several threads search at once).  Small host-pointer kNN calls hold the tree's
lock shared and run on pooled streams of their own, so threads search at the
same time; every row must equal the same query's row from one batched call."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_concurrent_single_point_searches(ikdg_mod):
    rng = np.random.default_rng(31)
    pts = rng.uniform(-20, 20, (200_000, 3)).astype(np.float32)
    tree = ikdg_mod.KDTree(0.5, 0.6, 0.2)
    tree.Build(pts)
    n_threads, per = 8, 400
    q = rng.uniform(-21, 21, (n_threads * per, 3)).astype(np.float32)
    want_ids, want_d2, want_xyz, _ = tree.knn(q, 5, 3.0)
    got = [None] * n_threads
    errors = []

    def worker(w):
        try:
            rows = []
            for i in range(w * per, (w + 1) * per):
                rows.append(tree.knn(q[i:i + 1], 5, 3.0))
            got[w] = rows
        except Exception as e:  # surfaced below
            errors.append(e)

    ts = [threading.Thread(target=worker, args=(w,)) for w in range(n_threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
    for w in range(n_threads):
        for j, (ids, d2, xyz, cnt) in enumerate(got[w]):
            i = w * per + j
            assert np.array_equal(ids[0], want_ids[i]), f"query {i}: ids differ"
            assert np.array_equal(d2[0].view(np.uint32), want_d2[i].view(np.uint32))
            assert np.array_equal(xyz[0].view(np.uint32), want_xyz[i].view(np.uint32))
    # a mutation between searches is seen by the next small search
    tree.Delete_Point_Boxes(np.array([[-100, -100, -100, 100, 100, 0]], np.float32))
    ids, d2, xyz, cnt = tree.knn(np.array([[0, 0, -5]], np.float32), 5)
    assert (xyz[0, :, 2] >= 0).all()
    tree.close()
