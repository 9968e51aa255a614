"""Comparison helpers shared by the oracle and GPU tests.

Golden fixtures hold the reference's own outputs (coordinates, no ids).  Where
several points lie at exactly the k-th distance the reference picks among them
by traversal order; these helpers then accept any of the tied points, and check
everything else bit for bit.
"""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, f"golden_{name}.npz"), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def bits(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, np.float32)).view(np.uint32)


def sorted_rows(xyz) -> np.ndarray:
    v = bits(np.asarray(xyz, np.float32).reshape(-1, 3))
    if len(v) == 0:
        return v.reshape(0, 3)
    return v[np.lexsort((v[:, 2], v[:, 1], v[:, 0]))]


def same_point_set(a, b) -> bool:
    return np.array_equal(sorted_rows(a), sorted_rows(b))


def sq_dist(q, p):
    q = np.asarray(q, np.float32)
    p = np.asarray(p, np.float32)
    dx, dy, dz = q[0] - p[..., 0], q[1] - p[..., 1], q[2] - p[..., 2]
    return (dx * dx + dy * dy) + dz * dz


def check_knn_rows(q, ref_xyz, ref_d2, ref_cnt, got_xyz, got_d2, got_cnt):
    """Raises AssertionError on the first query whose result differs."""
    for i in range(len(q)):
        c = int(ref_cnt[i])
        assert int(got_cnt[i]) == c, f"query {i}: count {got_cnt[i]} != {c}"
        if c == 0:
            continue
        rd, gd = bits(ref_d2[i, :c]), bits(got_d2[i, :c])
        assert np.array_equal(np.sort(rd), np.sort(gd)), f"query {i}: squared distances differ"
        last = np.float32(np.max(np.asarray(ref_d2[i, :c], np.float32)))
        rin = np.asarray(ref_d2[i, :c], np.float32) < last
        gin = np.asarray(got_d2[i, :c], np.float32) < last
        assert same_point_set(ref_xyz[i, :c][rin], got_xyz[i, :c][gin]), f"query {i}: neighbours differ"
        # points at the k-th distance: any tied point is acceptable, but it
        # must really sit at that distance
        tied = got_xyz[i, :c][~gin]
        assert np.all(bits(sq_dist(q[i], tied)) == bits(last)), f"query {i}: tie point at wrong distance"


def check_knn_rows_bulk(q, ref_xyz, ref_d2, ref_cnt, got_xyz, got_d2, got_cnt):
    """check_knn_rows for large batches: counts and distance bits are compared
    for all rows at once, points position by position in rows without two
    equal distances (both sides list a row in ascending distance), and the
    few rows with ties go through check_knn_rows."""
    ref_cnt = np.asarray(ref_cnt)
    assert np.array_equal(np.asarray(got_cnt), ref_cnt), "counts differ"
    k = np.asarray(ref_d2).shape[1]
    live = np.arange(k)[None, :] < ref_cnt[:, None]
    rd = np.where(live, bits(ref_d2), 0)
    gd = np.where(live, bits(got_d2), 0)
    bad = np.nonzero((rd != gd).any(1))[0]
    assert len(bad) == 0, f"squared distances differ in {len(bad)} rows, first {bad[:5]}"
    tie = (live[:, 1:] & (rd[:, 1:] == rd[:, :-1])).any(1)
    rx = np.where(live[..., None], bits(ref_xyz).reshape(live.shape + (3,)), 0)
    gx = np.where(live[..., None], bits(got_xyz).reshape(live.shape + (3,)), 0)
    bad = np.nonzero(~tie & (rx != gx).any((1, 2)))[0]
    assert len(bad) == 0, f"neighbours differ in {len(bad)} rows, first {bad[:5]}"
    rows = np.nonzero(tie)[0]
    if len(rows):
        check_knn_rows(np.asarray(q)[rows], np.asarray(ref_xyz)[rows], np.asarray(ref_d2)[rows], ref_cnt[rows],
                       np.asarray(got_xyz)[rows], np.asarray(got_d2)[rows], np.asarray(got_cnt)[rows])
    return len(rows)


def check_csr(ref_offs, ref_xyz, got_offs, got_xyz):
    assert np.array_equal(np.asarray(ref_offs, np.int64), np.asarray(got_offs, np.int64)), "hit counts differ"
    for i in range(len(ref_offs) - 1):
        a = ref_xyz[ref_offs[i]:ref_offs[i + 1]]
        b = got_xyz[got_offs[i]:got_offs[i + 1]]
        assert same_point_set(a, b), f"query {i}: hit sets differ"


class Adapter:
    """Uniform view of a tree implementation for fixture replay:
    knn -> (xyz, d2, cnt); box/radius -> (offsets, xyz); flatten -> xyz."""

    def __init__(self, tree, kind: str):
        self.t = tree
        self.kind = kind

    def knn(self, q, k, md=np.inf):
        if self.kind == "gpu":
            ids, d2, xyz, cnt = self.t.knn(q, k, md)
            return xyz, d2, cnt
        if self.kind == "spec":
            ids, d2 = self.t.knn(q, k, md)
            xyz = np.zeros(ids.shape + (3,), np.float32)
            lut = dict(zip(self.t.ids.tolist(), range(len(self.t.ids))))
            for idx in np.argwhere(ids >= 0):
                xyz[tuple(idx)] = self.t.pts[lut[int(ids[tuple(idx)])]]
            return xyz, d2, (ids >= 0).sum(1)
        return self.t.knn(q, k, md)

    def _csr_spec(self, lists):
        offs = np.zeros(len(lists) + 1, np.int64)
        offs[1:] = np.cumsum([len(x) for x in lists])
        lut = dict(zip(self.t.ids.tolist(), range(len(self.t.ids))))
        xyz = np.array([self.t.pts[lut[int(i)]] for x in lists for i in x], np.float32).reshape(-1, 3)
        return offs, xyz

    def box_search(self, b):
        if self.kind == "gpu":
            offs, ids, xyz = self.t.box_search(b)
            return offs, xyz
        if self.kind == "spec":
            return self._csr_spec(self.t.box_search(b))
        return self.t.box_search(b)

    def radius_search(self, c, r):
        if self.kind == "gpu":
            offs, ids, xyz = self.t.radius_search(c, r)
            return offs, xyz
        if self.kind == "spec":
            return self._csr_spec(self.t.radius_search(c, r))
        return self.t.radius_search(c, r)

    def flatten(self):
        if self.kind == "spec":
            return self.t.valid_points()[0]
        return self.t.flatten()

    def __getattr__(self, name):
        return getattr(self.t, name)


def replay_knn_fixture(make_tree):
    g = load("knn")
    t = make_tree(0.5, 0.6, 0.2)
    t.Build(g["pts"])
    for tag in ("k5", "k8_md05", "k1", "k20_md1"):
        xyz, d2, cnt = t.knn(g["q"], int(g[f"{tag}_k"]), float(g[f"{tag}_md"]))
        check_knn_rows(g["q"], g[f"{tag}_xyz"], g[f"{tag}_d2"], g[f"{tag}_cnt"], xyz, d2, cnt)
    check_csr(g["box_offs"], g["box_xyz"], *t.box_search(g["box"]))
    check_csr(g["rad_offs"], g["rad_xyz"], *t.radius_search(g["rad_c"], g["rad_r"]))
    assert t.validnum() == int(g["validnum"])
    assert np.array_equal(bits(t.tree_range()), bits(g["tree_range"])), "tree_range differs"


def replay_ops_fixture(make_tree):
    g = load("ops")
    t = make_tree(float(g["delete_param"]), float(g["balance_param"]), float(g["ds"]))
    t.Build(g["base"])
    for i in range(int(g["n_ops"])):
        kind = str(g[f"op{i}_kind"])
        data, ret = g[f"op{i}_data"], int(g[f"op{i}_ret"])
        if kind == "add":
            assert t.Add_Points(data, False) == ret
        elif kind == "del":
            t.Delete_Points(data)
        elif kind == "delbox":
            assert t.Delete_Point_Boxes(data) == ret, f"op {i}: Delete_Point_Boxes count"
        elif kind == "addds":
            assert t.Add_Points(data, True) == ret, f"op {i}: downsampled Add_Points count"
        elif kind == "validnum":
            assert t.validnum() == ret, f"op {i}: validnum"
    assert same_point_set(g["final_valid"], t.flatten())
    xyz, d2, cnt = t.knn(g["final_q"], 5)
    check_knn_rows(g["final_q"], g["final_xyz"], g["final_d2"], g["final_cnt"], xyz, d2, cnt)


def replay_downsample_fixture(make_tree):
    g = load("downsample")
    t = make_tree(0.5, 0.6, float(g["ds"]))
    t.Build(g["base"])
    for a, r in zip(g["adds"], g["rets"]):
        assert t.Add_Points(a, True) == int(r)
    assert t.validnum() == int(g["validnum"])
    assert same_point_set(g["final_valid"], t.flatten())


def replay_edge_fixture(make_tree):
    g = load("edge")
    t = make_tree(0.5, 0.6, 0.2)
    t.Build(g["small_pts"])
    xyz, d2, cnt = t.knn(g["small_q"], 5)
    check_knn_rows(g["small_q"], g["small_xyz"], g["small_d2"], g["small_cnt"], xyz, d2, cnt)
    xyz, d2, cnt = t.knn(g["small_q"], 5, 1.0)
    check_knn_rows(g["small_q"], g["small_md_xyz"], g["small_md_d2"], g["small_md_cnt"], xyz, d2, cnt)
    t = make_tree(0.5, 0.6, 0.2)
    t.Build(g["dup_pts"])
    xyz, d2, cnt = t.knn(g["dup_q"], 6)
    check_knn_rows(g["dup_q"], g["dup_xyz"], g["dup_d2"], g["dup_cnt"], xyz, d2, cnt)
    xyz, d2, cnt = t.knn(g["dup_pts"][:20], 3, 0.0)
    check_knn_rows(g["dup_pts"][:20], g["dup_md0_xyz"], g["dup_md0_d2"], g["dup_md0_cnt"], xyz, d2, cnt)
    t = make_tree(0.5, 0.6, 0.2)
    t.Build(np.zeros((0, 3), np.float32))
    xyz, d2, cnt = t.knn(np.zeros((1, 3), np.float32), 3)
    assert np.array_equal(cnt, g["empty_cnt"]) and t.size() == int(g["empty_size"])


def replay_restore_fixture(make_tree):
    """Add_Point_Boxes, acquire_removed_points, tree_range and root_alpha
    against the reference (see make_golden.restore_fixture for why these
    sequences do not depend on the reference's tree shape)."""
    g = load("restore")
    everything = np.array([[-1e9, -1e9, -1e9, 1e9, 1e9, 1e9]], np.float32)
    t = make_tree(0.5, 0.6, 0.2)
    t.Build(g["base"])
    assert np.array_equal(bits(t.tree_range()), bits(g["a_range_built"])), "tree_range after Build"
    assert t.Add_Points(g["a_dsadd"], True) == int(g["a_dsadd_ret"]), "downsampled insert count"
    t.Delete_Points(g["a_delpts"])
    assert t.Delete_Point_Boxes(g["a_slabs"]) == int(g["a_slab_ret"]), "slab deletion count"
    assert t.size() == int(g["a_size"]), "size(): a rebuild ran where the reference ran none"
    assert t.validnum() == int(g["a_validnum"])
    assert np.array_equal(bits(t.tree_range()), bits(g["a_range"])), "tree_range after deletions"
    bal, dele = t.root_alpha()
    # alpha_del = deleted / stored at the root: the same counts, the same
    # float division.  alpha_bal depends on the shape (the reference's root
    # holds one point of its own), so it is compared loosely.
    assert np.float32(dele) == np.float32(g["a_alpha"][1]), "root alpha_del"
    assert abs(bal - float(g["a_alpha"][0])) < 5e-3, "root alpha_bal"
    t.Add_Point_Boxes(everything)
    assert t.size() == int(g["a_restored_size"])
    assert t.validnum() == int(g["a_restored_validnum"]), "validnum after Add_Point_Boxes"
    assert same_point_set(g["a_restored_valid"], t.flatten()), "valid set after Add_Point_Boxes"
    assert len(t.acquire_removed_points()) == len(g["a_removed"]) == 0
    t = make_tree(0.0, 0.6, 0.2)
    t.Build(g["b_base"])
    assert t.Add_Points(g["b_dsadd"], True) == int(g["b_dsadd_ret"])
    t.Delete_Points(g["b_delpts"])
    assert t.Delete_Point_Boxes(g["b_boxes"]) == int(g["b_box_ret"])
    assert same_point_set(g["b_removed"], t.acquire_removed_points()), "acquire_removed_points multiset"
    assert len(t.acquire_removed_points()) == 0, "acquire_removed_points drains"
    assert t.size() == int(g["b_size"]) and t.validnum() == int(g["b_validnum"])
    assert same_point_set(g["b_valid"], t.flatten())
    assert np.array_equal(bits(t.tree_range()), bits(g["b_range"])), "tree_range after purges"
    assert np.float32(t.root_alpha()[1]) == np.float32(g["b_alpha"][1]) == 0


REPLAYS = [replay_knn_fixture, replay_ops_fixture, replay_downsample_fixture, replay_edge_fixture]
# Fixtures that need the whole tree API (the numpy model has no removed-point
# record or re-insertion): run against the port and the GPU library.
REPLAYS_TREE = REPLAYS + [replay_restore_fixture]
