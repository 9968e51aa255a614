"""GPU parity: libikdg (through its C ABI) against the brute-force oracle model.

Every comparison is bit-exact: point ids and float32 squared distances for kNN,
id sets for box / radius searches, id + coordinate sets of the valid points
after mutations.  Ties are broken by point id on both sides.
"""
import numpy as np
import pytest

import spec

pytestmark = pytest.mark.gpu


def canon_pts(xyz, ids):
    order = np.argsort(ids, kind="stable")
    return np.asarray(ids)[order], np.asarray(xyz, np.float32)[order]


def assert_same_valid(tree, ref):
    xyz, ids = tree.flatten(with_ids=True)
    rxyz, rids = ref.valid_points()
    a_ids, a_xyz = canon_pts(xyz, ids)
    b_ids, b_xyz = canon_pts(rxyz, rids)
    assert np.array_equal(a_ids, b_ids)
    assert np.array_equal(a_xyz.view(np.uint32), b_xyz.view(np.uint32))
    assert tree.validnum() == ref.validnum()


def assert_knn(tree, ref, q, k, max_dist=np.inf):
    ids, d2, xyz, cnt = tree.knn(q, k, max_dist)
    rid, rd2 = ref.knn(q, k, max_dist)
    assert np.array_equal(ids, rid), f"ids differ for k={k} max_dist={max_dist}"
    assert np.array_equal(d2.view(np.uint32), rd2.view(np.uint32))
    assert np.array_equal(cnt, (rid >= 0).sum(1))


def assert_ranges(tree, ref, boxes, centres, radii):
    offs, ids, _ = tree.box_search(boxes)
    for i, want in enumerate(ref.box_search(boxes)):
        assert np.array_equal(np.sort(ids[offs[i]:offs[i + 1]]), want)
    offs, ids, _ = tree.radius_search(centres, radii)
    for i, want in enumerate(ref.radius_search(centres, radii)):
        assert np.array_equal(np.sort(ids[offs[i]:offs[i + 1]]), want)


@pytest.mark.parametrize("lanes", [1, 2, 4])
def test_knn_every_list_storage(ikdg_mod, lanes):
    """k in registers (<= 16), in shared memory (17..64) and in the output
    rows (> 64), with 1, 2 and 4 lanes per query, with and without max_dist,
    plus the returned points and counts."""
    rng = np.random.default_rng(90 + lanes)
    pts = rng.uniform(-10, 10, (20000, 3)).astype(np.float32)
    pts[::97] = pts[1::97][: len(pts[::97])]  # exact duplicates: ties by id
    tree, ref = ikdg_mod.KDTree(), spec.SpecTree()
    tree.Build(pts)
    ref.Build(pts)
    tree.set_knn_lanes(lanes)
    q = rng.uniform(-11, 11, (700, 3)).astype(np.float32)
    for k in (3, 16, 17, 32, 48, 64, 65, 130):
        for md in (np.inf, 1.3):
            assert_knn(tree, ref, q, k, md)
            ids, d2, xyz, cnt = tree.knn(q, k, md)
            ok = ids >= 0
            assert np.array_equal(xyz[ok].view(np.uint32), pts[ids[ok]].view(np.uint32))


def test_snapshot_restore(ikdg_mod):
    """Map snapshot (flatten, ikd_Tree.cpp:1325-1352, as in the reference's
    async demo) and restore by Build: the snapshot is the model's valid set,
    and the restored tree answers like the original (points renumbered
    0..n-1 by Build) and like the model restored from the same snapshot."""
    rng = np.random.default_rng(31)
    pts = rng.uniform(-20, 20, (30000, 3)).astype(np.float32)
    a, ref = ikdg_mod.KDTree(0.5, 0.6, 0.3), spec.SpecTree(0.3)
    a.Build(pts)
    ref.Build(pts)
    add = rng.uniform(-20, 20, (5000, 3)).astype(np.float32)
    assert a.Add_Points(add, True) == ref.Add_Points(add, True)
    boxes = random_boxes(rng, 20, -20, 20, 1, 6)
    assert a.Delete_Point_Boxes(boxes) == ref.Delete_Point_Boxes(boxes)
    # the snapshot is the model's valid set, ids included
    assert_same_valid(a, ref)
    snap, ids = a.flatten(with_ids=True)
    b = ikdg_mod.KDTree(0.5, 0.6, 0.3)
    b.Build(snap)
    assert b.validnum() == a.validnum() == len(snap)
    q = rng.uniform(-21, 21, (2000, 3)).astype(np.float32)
    ia, da, xa, ca = a.knn(q, 8, 3.0)
    ib, db, xb, cb = b.knn(q, 8, 3.0)
    assert np.array_equal(ca, cb) and np.array_equal(da.view(np.uint32), db.view(np.uint32))
    ok = ia >= 0
    # same neighbours: map b's ids back through the snapshot order
    assert np.array_equal(ids[ib[ok]], ia[ok])
    # and the restored tree answers like the model restored from the snapshot
    rb = spec.SpecTree(0.3)
    rb.Build(snap)
    assert_knn(b, rb, q, 8, 3.0)


def random_boxes(rng, n, lo, hi, smin, smax):
    c = rng.uniform(lo, hi, (n, 3))
    s = rng.uniform(smin, smax, (n, 3))
    return np.concatenate([c - s / 2, c + s / 2], 1).astype(np.float32)


@pytest.mark.parametrize("n", [1, 17, 1000, 50000])
def test_knn_uniform(ikdg_mod, n):
    rng = np.random.default_rng(100 + n)
    pts = rng.uniform(-20, 20, (n, 3)).astype(np.float32)
    q = rng.uniform(-22, 22, (1500, 3)).astype(np.float32)
    tree, ref = ikdg_mod.KDTree(), spec.SpecTree()
    tree.Build(pts)
    ref.Build(pts)
    for k in (1, 5, 8, 16, 33):
        assert_knn(tree, ref, q, k)
    assert_knn(tree, ref, q, 5, 1.0)
    assert_knn(tree, ref, q, 3, 0.0)


def test_knn_ties_broken_by_id(ikdg_mod):
    # Integer lattice with duplicated points: many exactly equal distances.
    g = np.stack(np.meshgrid(*[np.arange(-6, 7)] * 3, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    pts = np.concatenate([g, g[::3]])
    q = np.concatenate([g[::7], g[::11] + 0.5]).astype(np.float32)
    tree, ref = ikdg_mod.KDTree(), spec.SpecTree()
    tree.Build(pts)
    ref.Build(pts)
    for k in (1, 4, 7, 20):
        assert_knn(tree, ref, q, k)


def test_box_and_radius(ikdg_mod):
    rng = np.random.default_rng(3)
    pts = rng.uniform(-10, 10, (30000, 3)).astype(np.float32)
    tree, ref = ikdg_mod.KDTree(), spec.SpecTree()
    tree.Build(pts)
    ref.Build(pts)
    boxes = random_boxes(rng, 200, -12, 12, 0.1, 8)
    cen = rng.uniform(-12, 12, (200, 3)).astype(np.float32)
    rad = rng.uniform(0.1, 5, 200).astype(np.float32)
    assert_ranges(tree, ref, boxes, cen, rad)
    # boxes snapped onto point coordinates exercise the half-open bounds
    sel = pts[rng.choice(len(pts), 50)]
    snapped = np.concatenate([sel, sel + 1.0], 1).astype(np.float32)
    assert_ranges(tree, ref, snapped, sel, np.float32(0.0))


def test_empty_tree(ikdg_mod):
    tree = ikdg_mod.KDTree()
    tree.Build(np.zeros((0, 3), np.float32))
    ids, d2, _, cnt = tree.knn(np.zeros((4, 3), np.float32), 3)
    assert (ids == -1).all() and np.isinf(d2).all() and (cnt == 0).all()
    assert tree.size() == 0 and tree.validnum() == 0
    offs, got, _ = tree.box_search(np.array([[-1, -1, -1, 1, 1, 1]], np.float32))
    assert offs[-1] == 0
    assert tree.Delete_Point_Boxes(np.array([[-1, -1, -1, 1, 1, 1]], np.float32)) == 0
    # Adding to an empty tree works (the reference dereferences a null root).
    pts = np.random.default_rng(0).uniform(-1, 1, (100, 3)).astype(np.float32)
    assert tree.Add_Points(pts, False) == 0
    ref = spec.SpecTree()
    ref.Build(np.zeros((0, 3), np.float32))
    ref.Add_Points(pts, False)
    assert_same_valid(tree, ref)
    assert_knn(tree, ref, pts[:20], 200)


def test_k_exceeds_valid_count(ikdg_mod):
    pts = np.array([[0, 0, 0], [1, 0, 0], [0, 2, 0]], np.float32)
    tree, ref = ikdg_mod.KDTree(), spec.SpecTree()
    tree.Build(pts)
    ref.Build(pts)
    assert_knn(tree, ref, np.array([[0.1, 0.1, 0]], np.float32), 5)
    assert_knn(tree, ref, np.array([[0.1, 0.1, 0]], np.float32), 5, 1.0)


def test_mutation_sequence(ikdg_mod):
    rng = np.random.default_rng(11)
    L = 8.0
    pts = rng.uniform(-L, L, (20000, 3)).astype(np.float32)
    tree, ref = ikdg_mod.KDTree(0.3, 0.6, 0.3), spec.SpecTree(0.3)
    tree.Build(pts)
    ref.Build(pts)
    q = rng.uniform(-L, L, (400, 3)).astype(np.float32)
    for it in range(8):
        add = rng.uniform(-L, L, (1500, 3)).astype(np.float32)
        assert tree.Add_Points(add, False) == ref.Add_Points(add, False) == 0
        cur, _ = ref.valid_points()
        dels = cur[rng.choice(len(cur), 300, replace=False)]
        tree.Delete_Points(dels)
        ref.Delete_Points(dels)
        boxes = random_boxes(rng, 3, -L, L, 0.5, 4)
        assert tree.Delete_Point_Boxes(boxes) == ref.Delete_Point_Boxes(boxes)
        add2 = rng.uniform(-L, L, (800, 3)).astype(np.float32)
        add2[:100] = cur[rng.choice(len(cur), 100)]
        assert tree.Add_Points(add2, True) == ref.Add_Points(add2, True)
        assert_same_valid(tree, ref)
        assert_knn(tree, ref, q, 5)
        assert_knn(tree, ref, q, 12, 1.2)
    assert_ranges(tree, ref, random_boxes(rng, 50, -L, L, 0.5, 6), q[:50], np.float32(1.5))


@pytest.mark.parametrize("ds", [0.2, 0.5, 0.37])
def test_downsample(ikdg_mod, ds):
    rng = np.random.default_rng(int(ds * 100))
    base = rng.uniform(-5, 5, (8000, 3)).astype(np.float32)
    tree, ref = ikdg_mod.KDTree(0.5, 0.6, ds), spec.SpecTree(ds)
    tree.Build(base)
    ref.Build(base)
    for it in range(4):
        # dense clusters: many new points per voxel, exact duplicates included
        c = rng.uniform(-5, 5, (40, 3))
        add = (c[rng.integers(0, 40, 3000)] + rng.normal(0, ds, (3000, 3))).astype(np.float32)
        add[::17] = add[::17][::-1]
        add[5::29] = base[rng.choice(len(base), len(add[5::29]))]
        assert tree.Add_Points(add, True) == ref.Add_Points(add, True)
        assert_same_valid(tree, ref)
    assert_knn(tree, ref, rng.uniform(-5, 5, (300, 3)).astype(np.float32), 5)


def test_downsample_deletion_walk_when_pair_list_overflows(ikdg_mod, monkeypatch):
    # The voxels' stored points are deleted from the (voxel, point) list the
    # searches wrote; when that list overflows, a walk of every voxel box
    # does it instead.  A room of 8 pairs forces the walk.
    monkeypatch.setenv("IKDG_DS_PAIR_CAP", "8")
    rng = np.random.default_rng(47)
    base = rng.uniform(-4, 4, (6000, 3)).astype(np.float32)
    tree, ref = ikdg_mod.KDTree(0.5, 0.6, 0.3), spec.SpecTree(0.3)
    tree.Build(base)
    ref.Build(base)
    for it in range(3):
        add = rng.uniform(-4, 4, (2500, 3)).astype(np.float32)
        assert tree.Add_Points(add, True) == ref.Add_Points(add, True)
        assert_same_valid(tree, ref)


def test_downsample_voxel_boundaries(ikdg_mod):
    # Coordinates exactly on voxel faces and a 1-ulp neighbourhood of them.
    ds = 0.2
    k = np.arange(-20, 20, dtype=np.float32)
    faces = (k * np.float32(ds)).astype(np.float32)
    vals = np.concatenate([faces, np.nextafter(faces, np.float32(np.inf)), np.nextafter(faces, -np.float32(np.inf))])
    rng = np.random.default_rng(5)
    add = rng.choice(vals, (4000, 3)).astype(np.float32)
    base = rng.choice(vals, (2000, 3)).astype(np.float32)
    tree, ref = ikdg_mod.KDTree(0.5, 0.6, ds), spec.SpecTree(ds)
    tree.Build(base)
    ref.Build(base)
    assert tree.Add_Points(add, True) == ref.Add_Points(add, True)
    assert_same_valid(tree, ref)


def test_downsample_dense_voxels(ikdg_mod):
    # Hundreds of new points in one voxel (the long hash runs folded by a warp)
    # with 0, 1 and 3 stored points, a stored point at the exact centre that
    # only coincident points can displace, distance ties between new points
    # (the later one wins) and exact duplicates, interleaved in input order.
    ds = np.float32(0.5)
    rng = np.random.default_rng(41)

    def in_voxel(cell, m):
        lo = np.asarray(cell, np.float32) * ds
        return (lo + rng.uniform(0.01, 0.49, (m, 3))).astype(np.float32)

    centre4 = (np.asarray([-30, 8, 2], np.float32) * ds + ds / 2).astype(np.float32)
    base = np.concatenate([rng.uniform(-5, 5, (3000, 3)).astype(np.float32),
                           in_voxel((30, 30, 30), 1), in_voxel((-30, 30, 30), 3), centre4[None]])
    tree, ref = ikdg_mod.KDTree(0.5, 0.6, float(ds)), spec.SpecTree(float(ds))
    tree.Build(base)
    ref.Build(base)
    for it in range(2):
        # one ulp off the stored centre point: farther from the centre but the
        # same point (|a - b| < 1e-6), so the stored point stays the winner
        nudged = np.nextafter(centre4, np.float32(np.inf))[None].repeat(30, 0)
        parts = [in_voxel((40, 40, 40), 900), in_voxel((30, 30, 30), 700), in_voxel((-30, 30, 30), 600),
                 np.repeat(centre4[None], 40, 0), nudged, in_voxel((-30, 8, 2), 300)]
        # mirrored pairs about the centre of voxel (40, 40, 40): equal distances
        c1 = (np.asarray([40, 40, 40], np.float32) * ds + ds / 2).astype(np.float32)
        off = rng.uniform(0.01, 0.2, (100, 3)).astype(np.float32)
        parts += [c1 + off, c1 - off]
        add = np.concatenate(parts)
        add = np.concatenate([add, add[rng.choice(len(add), 200)]])  # exact duplicates
        add = add[rng.permutation(len(add))]
        assert tree.Add_Points(add, True) == ref.Add_Points(add, True)
        assert_same_valid(tree, ref)


def test_downsample_dense_voxel_split_by_slivers(ikdg_mod):
    # A voxel with hundreds of new points whose run is cut into several
    # sub-batches by points on voxel faces (one ulp either side), which are
    # folded alone: the warp fold must stop at each sub-batch end and resume.
    ds = np.float32(0.2)
    rng = np.random.default_rng(43)
    lo = np.asarray([7, -3, 2], np.float32) * ds
    dense = (lo + rng.uniform(0.005, 0.195, (700, 3))).astype(np.float32)
    # coordinates near voxel faces whose float voxel box misses them or whose
    # neighbour's box also holds them (the library folds such points alone)
    k = np.arange(-200, 200, dtype=np.float32)
    faces = (k * ds).astype(np.float32)
    near = np.concatenate([faces, np.nextafter(faces, np.float32(np.inf)), np.nextafter(faces, -np.float32(np.inf))])

    def in_box(c, f):
        b_lo = np.float32(f * ds)
        return (b_lo <= c) & (c < np.float32(b_lo + ds))

    f = np.floor(near / ds).astype(np.float32)
    sliver = ~in_box(near, f) | in_box(near, f - 1) | in_box(near, f + 1)
    assert sliver.sum() > 20
    slivers = np.stack([rng.choice(near[sliver], 12), rng.uniform(-1, 1, 12), rng.uniform(-1, 1, 12)], 1)
    slivers = slivers.astype(np.float32)
    add = dense.copy()
    cut = np.sort(rng.choice(np.arange(50, 650), 12, replace=False))
    add = np.insert(add, cut, slivers, axis=0)
    base = np.concatenate([rng.uniform(-1, 2, (1500, 3)).astype(np.float32), dense[:2] + np.float32(0.001)])
    tree, ref = ikdg_mod.KDTree(0.5, 0.6, float(ds)), spec.SpecTree(float(ds))
    tree.Build(base)
    ref.Build(base)
    for it in range(2):
        assert tree.Add_Points(add, True) == ref.Add_Points(add, True)
        assert_same_valid(tree, ref)
        add = add[rng.permutation(len(add))]


def test_growth_and_rebalance(ikdg_mod):
    # All inserts land in one corner: leaf overflow splits, scapegoat rebuilds,
    # pool growth.
    rng = np.random.default_rng(9)
    base = rng.uniform(-50, 50, (5000, 3)).astype(np.float32)
    tree, ref = ikdg_mod.KDTree(0.5, 0.6, 0.2), spec.SpecTree(0.2)
    tree.Build(base)
    ref.Build(base)
    for it in range(6):
        add = rng.uniform(40, 50, (20000, 3)).astype(np.float32)
        tree.Add_Points(add, False)
        ref.Add_Points(add, False)
    assert_same_valid(tree, ref)
    q = rng.uniform(-50, 50, (500, 3)).astype(np.float32)
    assert_knn(tree, ref, q, 10)
    box = np.array([[30, 30, 30, 50, 50, 50]], np.float32)
    assert tree.Delete_Point_Boxes(box) == ref.Delete_Point_Boxes(box)
    assert_same_valid(tree, ref)
    assert_knn(tree, ref, q, 10)
    tree.rebuild()
    assert tree.size() == tree.validnum()
    assert_knn(tree, ref, q, 10)


def test_knn_binned_batches_match(ikdg_mod):
    # Batches of >= 2048 queries are reordered by k-d cell before the search;
    # results must be identical to small (unbinned) batches and the model.
    rng = np.random.default_rng(21)
    pts = rng.uniform(-30, 30, (200000, 3)).astype(np.float32)
    q = rng.uniform(-31, 31, (12000, 3)).astype(np.float32)
    tree = ikdg_mod.KDTree()
    tree.Build(pts)
    for k, md in ((5, np.inf), (9, 1.5), (70, np.inf)):
        ids, d2, xyz, cnt = tree.knn(q, k, md)
        for lo in range(0, len(q), 1000):
            i2, d22, x2, c2 = tree.knn(q[lo:lo + 1000], k, md)
            assert np.array_equal(ids[lo:lo + 1000], i2) and np.array_equal(d2[lo:lo + 1000], d22)
            assert np.array_equal(xyz[lo:lo + 1000], x2) and np.array_equal(cnt[lo:lo + 1000], c2)
    ref = spec.SpecTree()
    ref.Build(pts)
    sub = q[:3000]
    ids, d2, _, _ = tree.knn(sub, 5)
    rid, rd2 = ref.knn(sub, 5)
    assert np.array_equal(ids, rid) and np.array_equal(d2, rd2)


def test_host_direct_and_staged_paths_agree(ikdg_mod, monkeypatch):
    # Where the GPU can address pageable host memory the host-pointer search
    # runs directly on the caller's buffers; IKDG_HOST_STAGING=1 forces the
    # copy path.  Both must give identical results.
    rng = np.random.default_rng(31)
    pts = rng.uniform(-10, 10, (50000, 3)).astype(np.float32)
    q = rng.uniform(-10, 10, (30000, 3)).astype(np.float32)
    direct = ikdg_mod.KDTree()
    monkeypatch.setenv("IKDG_HOST_STAGING", "1")
    staged = ikdg_mod.KDTree()
    monkeypatch.delenv("IKDG_HOST_STAGING")
    for t in (direct, staged):
        t.Build(pts)
    for k, md in ((5, np.inf), (11, 0.8)):
        a = direct.knn(q, k, md)
        b = staged.knn(q, k, md)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("downsample", [False, True])
def test_non_finite_input_rejected_without_change(ikdg_mod, downsample):
    """A batch with a non-finite coordinate is refused with IKDG_BAD_ARG and
    leaves the tree as it was (valid set, size, and the ids of later
    insertions)."""
    rng = np.random.default_rng(55)
    pts = rng.uniform(-5, 5, (5000, 3)).astype(np.float32)
    tree, ref = ikdg_mod.KDTree(0.5, 0.6, 0.3), spec.SpecTree(0.3)
    tree.Build(pts)
    ref.Build(pts)
    bad = rng.uniform(-5, 5, (300, 3)).astype(np.float32)
    bad[123, 1] = np.nan
    size0 = tree.size()
    with pytest.raises(ikdg_mod.IkdgError) as e:
        tree.Add_Points(bad, downsample)
    assert e.value.status == ikdg_mod.BAD_ARG
    assert tree.size() == size0
    assert_same_valid(tree, ref)
    good = rng.uniform(-5, 5, (300, 3)).astype(np.float32)
    assert tree.Add_Points(good, downsample) == ref.Add_Points(good, downsample)
    assert_same_valid(tree, ref)
    assert tree.validate() == 0
    tree.close()
