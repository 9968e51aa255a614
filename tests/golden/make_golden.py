"""Generates the golden fixtures in this directory by running the UNMODIFIED
ikd-Tree reference (oracle/_ref/libikd_ref.so, built by `make -C oracle ref`
from the reference checkout) on small seeded inputs.

The reference ships no tests or golden vectors of its own, so these fixtures are
the pin: the oracle port, the numpy model and the GPU library are all checked
against them.  Regenerate with:  python tests/golden/make_golden.py [names]
(needs the reference library built from the reference sources; the GPU
tests only read the .npz files).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))
import oracle_lib  # noqa: E402

F32 = np.float32


def boxes(rng, n, lo, hi, smin, smax):
    c = rng.uniform(lo, hi, (n, 3))
    s = rng.uniform(smin, smax, (n, 3))
    return np.concatenate([c - s / 2, c + s / 2], 1).astype(F32)


def knn_fixture():
    rng = np.random.default_rng(11)
    pts = rng.uniform(-5, 5, (4000, 3)).astype(F32)
    q = rng.uniform(-5.5, 5.5, (300, 3)).astype(F32)
    t = oracle_lib.OracleTree(0.5, 0.6, 0.2, kind="ref")
    t.Build(pts)
    out = {"pts": pts, "q": q}
    for tag, k, md in (("k5", 5, np.inf), ("k8_md05", 8, 0.5), ("k1", 1, np.inf), ("k20_md1", 20, 1.0)):
        xyz, d2, cnt = t.knn(q, k, md)
        out[f"{tag}_xyz"], out[f"{tag}_d2"], out[f"{tag}_cnt"] = xyz, d2, cnt
        out[f"{tag}_k"] = np.int32(k)
        out[f"{tag}_md"] = np.float64(md)
    bx = boxes(rng, 30, -5, 5, 0.5, 3)
    offs, xyz = t.box_search(bx)
    out.update(box=bx, box_offs=offs, box_xyz=xyz)
    rc = rng.uniform(-5, 5, (30, 3)).astype(F32)
    rr = rng.uniform(0.3, 1.5, 30).astype(F32)
    offs, xyz = t.radius_search(rc, rr)
    out.update(rad_c=rc, rad_r=rr, rad_offs=offs, rad_xyz=xyz)
    out["size"] = np.int64(t.size())
    out["validnum"] = np.int64(t.validnum())
    out["tree_range"] = t.tree_range()
    t.close()
    return out


def ops_fixture():
    """A mixed sequence; records every return value and the final valid set."""
    rng = np.random.default_rng(12)
    L = 5.0
    base = rng.uniform(-L, L, (3000, 3)).astype(F32)
    t = oracle_lib.OracleTree(0.3, 0.6, 0.3, kind="ref")
    t.Build(base)
    out = {"base": base, "ds": np.float32(0.3), "delete_param": np.float32(0.3), "balance_param": np.float32(0.6)}
    ops = []
    for it in range(5):
        a = rng.uniform(-L, L, (300, 3)).astype(F32)
        ops.append(("add", a, t.Add_Points(a, False)))
        cur = t.flatten()
        d = cur[rng.choice(len(cur), 60, replace=False)]
        t.Delete_Points(d)
        ops.append(("del", d, 0))
        b = boxes(rng, 3, -L, L, 0.5, 2.5)
        ops.append(("delbox", b, t.Delete_Point_Boxes(b)))
        a2 = rng.uniform(-L, L, (400, 3)).astype(F32)
        a2[:40] = cur[rng.choice(len(cur), 40)]
        ops.append(("addds", a2, t.Add_Points(a2, True)))
        ops.append(("validnum", np.zeros((0, 3), F32), t.validnum()))
    for i, (kind, data, ret) in enumerate(ops):
        out[f"op{i}_kind"] = np.array(kind)
        out[f"op{i}_data"] = data
        out[f"op{i}_ret"] = np.int64(ret)
    out["n_ops"] = np.int64(len(ops))
    out["final_valid"] = t.flatten()
    q = rng.uniform(-L, L, (200, 3)).astype(F32)
    xyz, d2, cnt = t.knn(q, 5)
    out.update(final_q=q, final_xyz=xyz, final_d2=d2, final_cnt=cnt)
    t.close()
    return out


def planar_points(rng, n):
    """Ground plane plus a few vertical walls with 2 cm noise (LiDAR-like)."""
    g = np.c_[rng.uniform(-20, 20, (n // 2, 2)), np.zeros(n // 2)]
    walls = []
    for _ in range(6):
        c = rng.uniform(-15, 15, 2)
        yaw = rng.uniform(0, np.pi)
        ln, ht = rng.uniform(3, 15), rng.uniform(2, 6)
        m = (n - n // 2) // 6
        s = rng.uniform(-ln / 2, ln / 2, m)
        h = rng.uniform(0, ht, m)
        walls.append(np.c_[c[0] + s * np.cos(yaw), c[1] + s * np.sin(yaw), h])
    p = np.concatenate([g] + walls)
    return (p + rng.normal(0, 0.02, p.shape)).astype(F32)


def downsample_fixture():
    rng = np.random.default_rng(13)
    base = planar_points(rng, 6000)
    t = oracle_lib.OracleTree(0.5, 0.6, 0.5, kind="ref")
    t.Build(base)
    adds = [planar_points(rng, 3000) for _ in range(3)]
    rets = [t.Add_Points(a, True) for a in adds]
    out = {"base": base, "ds": np.float32(0.5), "adds": np.stack(adds), "rets": np.array(rets, np.int64),
           "final_valid": t.flatten(), "validnum": np.int64(t.validnum())}
    t.close()
    return out


def edge_fixture():
    out = {}
    # three points, k larger than the tree
    t = oracle_lib.OracleTree(kind="ref")
    p3 = np.array([[0, 0, 0], [1, 0, 0], [0, 2, 0]], F32)
    t.Build(p3)
    q = np.array([[0.1, 0.1, 0.0], [5, 5, 5]], F32)
    xyz, d2, cnt = t.knn(q, 5)
    out.update(small_pts=p3, small_q=q, small_xyz=xyz, small_d2=d2, small_cnt=cnt)
    xyz, d2, cnt = t.knn(q, 5, 1.0)
    out.update(small_md_xyz=xyz, small_md_d2=d2, small_md_cnt=cnt)
    t.close()
    # duplicated points (exact distance ties) and a zero max_dist
    rng = np.random.default_rng(14)
    g = rng.integers(-3, 4, (500, 3)).astype(F32)
    t = oracle_lib.OracleTree(kind="ref")
    t.Build(g)
    q = rng.integers(-3, 4, (50, 3)).astype(F32) + F32(0.25)
    xyz, d2, cnt = t.knn(q, 6)
    out.update(dup_pts=g, dup_q=q, dup_xyz=xyz, dup_d2=d2, dup_cnt=cnt)
    xyz, d2, cnt = t.knn(g[:20], 3, 0.0)
    out.update(dup_md0_xyz=xyz, dup_md0_d2=d2, dup_md0_cnt=cnt)
    t.close()
    # empty tree: Build with no points, then a search
    t = oracle_lib.OracleTree(kind="ref")
    t.Build(np.zeros((0, 3), F32))
    xyz, d2, cnt = t.knn(np.zeros((1, 3), F32), 3)
    out.update(empty_cnt=cnt, empty_size=np.int64(t.size()))
    t.close()
    return out


def restore_fixture():
    """Add_Point_Boxes, acquire_removed_points, tree_range and root_alpha
    (ikd_Tree.cpp:491-511, :762-815, :558-571, :99-126, :148-165).

    Both phases are laid out so that the reference's result does not depend on
    its tree shape:
    * phase A (delete_param 0.5): a downsampled insertion that
      downsample-deletes about half of 300 stored points, then sparse point
      deletions and thin slab deletions; nothing is dense enough to trigger a
      rebuild (size() stays the number of stored points), so every deleted
      point is still stored when one box covering all space restores them.
      Points removed by downsampling stay deleted.
    * phase B (delete_param 0, a tree of 1,400 points, so that every rebuild
      runs inline): every subtree that holds a deleted point violates the
      delete criterion, so rebuilds purge every deleted point and
      acquire_removed_points returns all point- and box-deleted ones (not the
      downsample-deleted ones)."""
    rng = np.random.default_rng(16)  # a seed whose phase A runs no rebuild in the reference
    L = 50.0
    base = rng.uniform(-L, L, (100000, 3)).astype(F32)
    out = {"base": base}
    t = oracle_lib.OracleTree(0.5, 0.6, 0.2, kind="ref")
    t.Build(base)
    out["a_range_built"] = t.tree_range()
    # (root_alpha right after Build is not recorded: BuildTree never sets the
    # root's alpha fields, ikd_Tree.cpp:573-622, so they hold whatever the
    # allocation held)
    # the downsampled insertion comes first: with no deleted point in the
    # tree yet, the reference's lazy subtree flags cannot carry the
    # downsample mark onto points deleted earlier (which depends on its shape)
    near = base[rng.choice(len(base), 300, replace=False)] + F32(0.001)
    out["a_dsadd"] = near.astype(F32)
    out["a_dsadd_ret"] = np.int64(t.Add_Points(near.astype(F32), True))
    dp = base[rng.choice(len(base), 1500, replace=False)]
    t.Delete_Points(dp)
    xs = rng.uniform(-L, L, 4)
    slabs = np.array([[x, -100, -100, x + 0.3, 100, 100] for x in xs], F32)
    out["a_delpts"], out["a_slabs"] = dp, slabs
    out["a_slab_ret"] = np.int64(t.Delete_Point_Boxes(slabs))
    out["a_size"] = np.int64(t.size())
    out["a_validnum"] = np.int64(t.validnum())
    out["a_range"] = t.tree_range()
    out["a_alpha"] = np.array(t.root_alpha(), F32)
    everything = np.array([[-1e9, -1e9, -1e9, 1e9, 1e9, 1e9]], F32)
    t.Add_Point_Boxes(everything)
    out["a_restored_size"] = np.int64(t.size())
    out["a_restored_validnum"] = np.int64(t.validnum())
    out["a_restored_valid"] = t.flatten()
    out["a_removed"] = t.acquire_removed_points()
    # phase B: a tree below the reference's background-rebuild size (1,500
    # points, ikd_Tree.h:15), so every rebuild runs inline and the result
    # does not depend on thread timing
    t.close()
    base_b = rng.uniform(-10, 10, (1400, 3)).astype(F32)
    out["b_base"] = base_b
    t = oracle_lib.OracleTree(0.0, 0.6, 0.2, kind="ref")
    t.Build(base_b)
    near_b = base_b[rng.choice(len(base_b), 60, replace=False)] + F32(0.001)
    out["b_dsadd"] = near_b.astype(F32)
    out["b_dsadd_ret"] = np.int64(t.Add_Points(near_b.astype(F32), True))
    cur = t.flatten()
    dpb = cur[rng.choice(len(cur), 100, replace=False)]
    t.Delete_Points(dpb)
    bb = boxes(rng, 2, -10, 10, 4, 8)
    out["b_delpts"], out["b_boxes"] = dpb, bb
    out["b_box_ret"] = np.int64(t.Delete_Point_Boxes(bb))
    out["b_removed"] = t.acquire_removed_points()
    out["b_size"] = np.int64(t.size())
    out["b_validnum"] = np.int64(t.validnum())
    out["b_valid"] = t.flatten()
    out["b_range"] = t.tree_range()
    out["b_alpha"] = np.array(t.root_alpha(), F32)
    t.close()
    assert out["a_size"] == len(base) + out["a_dsadd_ret"], "phase A triggered a rebuild"
    assert out["b_size"] == out["b_validnum"], "phase B left deleted points stored"
    return out


def main():
    if not oracle_lib.available("ref"):
        oracle_lib.build("ref")
    only = sys.argv[1:]
    for name, fn in (("knn", knn_fixture), ("ops", ops_fixture), ("downsample", downsample_fixture),
                     ("edge", edge_fixture), ("restore", restore_fixture)):
        if only and name not in only:
            continue
        data = fn()
        np.savez_compressed(os.path.join(HERE, f"golden_{name}.npz"), **data)
        print("wrote", name, sum(v.nbytes for v in data.values() if hasattr(v, "nbytes")), "bytes")


if __name__ == "__main__":
    main()
