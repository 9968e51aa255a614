"""Multi-tree batches (one graph launch) against the per-call device path.

Every request of a batch must give exactly what the same request gives
through the per-call entry points (ikdg_knn_device, ikdg_box_search_device,
ikdg_radius_search_device) on the same tree: kNN ids, squared distances,
points and counts, and the box / radius CSR offsets, ids and points, bit for
bit.  The per-call path itself is pinned to the oracle elsewhere; a kNN, a
box and a radius request are also checked against the numpy model here.
Covered: all kNN register classes and lanes values, an empty tree, trees
mutated (pools grown) between runs of the same graph, runs without a graph,
queries in Morton order and in the given order, a capacity overflow, and the
autotuner.
"""
import math

import numpy as np
import pytest

import synthetic as S
from spec import SpecTree

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

DEV = "cuda:0"


def t32(a, dtype=torch.float32):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV, dtype)


class Req:
    """Device buffers of one request, with a per-call rerun for comparison."""

    def __init__(self, kind, tree, maps_entry, **kw):
        self.kind, self.tree = kind, tree
        self.__dict__.update(kw)

    @staticmethod
    def knn(tree, q, k, max_dist):
        r = Req("knn", tree, None, k=k, max_dist=max_dist, nq=len(q))
        r.q = t32(q)
        n = max(len(q), 1)
        r.ids = torch.full((n, k), -7, dtype=torch.int32, device=DEV)
        r.d2 = torch.full((n, k), -7.0, dtype=torch.float32, device=DEV)
        r.xyz = torch.full((n, k, 3), -7.0, dtype=torch.float32, device=DEV)
        r.cnt = torch.full((n,), -7, dtype=torch.int32, device=DEV)
        return r

    @staticmethod
    def rng(kind, tree, q, radius=None, capacity=None):
        r = Req(kind, tree, None, nq=len(q))
        r.q = t32(q)
        r.radius = t32(radius) if radius is not None else None
        r.offsets = torch.full((len(q) + 1,), -7, dtype=torch.int64, device=DEV)
        r.total = torch.zeros((1,), dtype=torch.int64, device=DEV)
        r.capacity = capacity
        return r

    def size_range(self, headroom=False):
        """Runs the per-call count to size the outputs (capacity = total, or
        room for growth)."""
        self.call(self.tree, count_only=True)
        torch.cuda.synchronize()
        tot = int(self.total.item())
        if self.capacity is None:
            self.capacity = 2 * tot + 4096 if headroom else tot
        self.ids = torch.full((max(self.capacity, 1),), -7, dtype=torch.int32, device=DEV)
        self.xyz = torch.full((max(self.capacity, 1), 3), -7.0, dtype=torch.float32, device=DEV)
        return tot

    def add_to(self, b):
        if self.kind == "knn":
            return b.add_knn(self.tree, self.q.data_ptr(), self.nq, self.k, self.max_dist, self.ids.data_ptr(),
                             self.d2.data_ptr(), self.xyz.data_ptr(), self.cnt.data_ptr())
        if self.kind == "box":
            return b.add_box_search(self.tree, self.q.data_ptr(), self.nq, self.offsets.data_ptr(),
                                    self.ids.data_ptr(), self.capacity, self.xyz.data_ptr())
        return b.add_radius_search(self.tree, self.q.data_ptr(), self.nq, self.radius.data_ptr(),
                                   self.offsets.data_ptr(), self.ids.data_ptr(), self.capacity, self.xyz.data_ptr())

    def outputs(self):
        torch.cuda.synchronize()
        if self.kind == "knn":
            n = self.nq
            return [x[:n].cpu().numpy().copy() for x in (self.ids, self.d2, self.xyz, self.cnt)]
        off = self.offsets.cpu().numpy().copy()
        m = int(off[-1]) if self.nq else 0
        m = min(m, self.capacity)
        return [off, self.ids[:m].cpu().numpy().copy(), self.xyz[:m].cpu().numpy().copy()]

    def call(self, tree, count_only=False):
        """The same request through the per-call device entry point."""
        if self.kind == "knn":
            tree.knn_device(self.q.data_ptr(), self.nq, self.k, self.max_dist, self.ids.data_ptr(),
                            self.d2.data_ptr(), self.xyz.data_ptr(), self.cnt.data_ptr())
        elif self.kind == "box":
            tree.box_search_device(self.q.data_ptr(), self.nq, self.offsets.data_ptr(),
                                   0 if count_only else self.ids.data_ptr(), 0 if count_only else self.capacity,
                                   0 if count_only else self.xyz.data_ptr(), self.total.data_ptr())
        else:
            tree.radius_search_device(self.q.data_ptr(), self.nq, self.radius.data_ptr(), self.offsets.data_ptr(),
                                      0 if count_only else self.ids.data_ptr(), 0 if count_only else self.capacity,
                                      0 if count_only else self.xyz.data_ptr(), self.total.data_ptr())
        tree.synchronize()

    def clobber(self):
        for name in ("ids", "d2", "xyz", "cnt", "offsets"):
            if hasattr(self, name) and getattr(self, name) is not None:
                getattr(self, name).fill_(-7)


def per_call(reqs):
    out = []
    for r in reqs:
        r.clobber()
        r.call(r.tree)
        out.append(r.outputs())
    return out


def batched(b, reqs):
    for r in reqs:
        r.clobber()
    b.run()
    b.synchronize(sum(r.kind != "knn" for r in reqs))
    return [r.outputs() for r in reqs]


def assert_same_sets(a, b, reqs):
    """Same results up to the order of hits within a query (for trees of
    different shapes): kNN rows exactly, range offsets exactly and each
    query's (id, point) set."""
    for i, (x, y) in enumerate(zip(a, b)):
        if reqs[i].kind == "knn":
            assert_same([x], [y], [reqs[i]])
            continue
        (oa, ia, pa), (ob, ib, pb) = x, y
        assert np.array_equal(oa, ob), f"request {i}: offsets differ"
        for qi in range(len(oa) - 1):
            s = slice(oa[qi], oa[qi + 1])
            ka, kb = np.argsort(ia[s], kind="stable"), np.argsort(ib[s], kind="stable")
            assert np.array_equal(ia[s][ka], ib[s][kb]), f"request {i} query {qi}: ids differ"
            assert np.array_equal(pa[s][ka].view(np.uint32), pb[s][kb].view(np.uint32)), \
                f"request {i} query {qi}: points differ"


def assert_same(a, b, reqs):
    for i, (x, y) in enumerate(zip(a, b)):
        for j, (u, v) in enumerate(zip(x, y)):
            assert u.shape == v.shape and np.array_equal(u.view(np.uint8), v.view(np.uint8)), \
                f"request {i} ({reqs[i].kind}) output {j} differs"


def make_scene(ikdg_mod, seed, n_maps, headroom=False):
    maps = S.multi_maps(seed, n_maps=n_maps, size_range=(2e3, 2e5), query_range=(300, 5000), kmax=16)
    trees = []
    for m in maps:
        t = ikdg_mod.KDTree(0.5, 0.6, 0.5)
        t.Build(m.points)
        trees.append(t)
    empty = ikdg_mod.KDTree(0.5, 0.6, 0.5)
    reqs = []
    ks = [1, 2, 3, 4, 5, 8, 11, 16]
    for i, (m, t) in enumerate(zip(maps, trees)):
        k = ks[i % len(ks)]
        reqs.append(Req.knn(t, m.knn_q, k, m.max_dist if i % 3 else math.inf))
        reqs.append(Req.rng("box", t, m.boxes))
        reqs.append(Req.rng("radius", t, m.radius_q, m.radius))
    m0 = maps[0]
    reqs.append(Req.knn(empty, m0.knn_q[:50], 4, math.inf))
    reqs.append(Req.rng("box", empty, m0.boxes[:20]))
    reqs.append(Req.knn(trees[1], m0.knn_q[:0], 3, 1.0))       # no queries
    reqs.append(Req.rng("radius", trees[1], m0.radius_q[:0], m0.radius[:0]))
    for r in reqs:
        if r.kind != "knn":
            r.size_range(headroom)
    b = ikdg_mod.Batch()
    lanes = [0, 1, 2, 4]
    for i, r in enumerate(reqs):
        idx = r.add_to(b)
        if r.kind == "knn":
            b.set_knn_lanes(idx, lanes[i % 4])
    return maps, trees, empty, reqs, b


@pytest.fixture(scope="module")
def scene(ikdg_mod):
    return make_scene(ikdg_mod, 3101, 7)


def test_batch_matches_per_call(scene):
    maps, trees, empty, reqs, b = scene
    ref = per_call(reqs)
    got = batched(b, reqs)
    assert_same(got, ref, reqs)
    # a second run of the same graph
    got2 = batched(b, reqs)
    assert_same(got2, ref, reqs)
    # without a graph
    b.set_graph(False)
    got3 = batched(b, reqs)
    b.set_graph(True)
    assert_same(got3, ref, reqs)


def test_batch_knn_matches_oracle(scene):
    maps, trees, empty, reqs, b = scene
    r = reqs[0]
    batched(b, reqs)
    ids, d2, xyz, cnt = r.outputs()
    spec = SpecTree()
    spec.Build(maps[0].points)
    sid, sd2 = spec.knn(maps[0].knn_q, r.k, r.max_dist)
    assert np.array_equal(ids, sid) and np.array_equal(d2.view(np.uint32), sd2.view(np.uint32))


def test_batch_query_order_changes_nothing(scene):
    """Every request's queries searched in Morton order and in the given
    order (the default): the same bytes as the per-call path."""
    maps, trees, empty, reqs, b = scene
    ref = per_call(reqs)
    for ordered in (True, False):
        b.set_query_order(ordered)
        assert_same(batched(b, reqs), ref, reqs)


def test_batch_range_requests_match_oracle(scene):
    """A box and a radius request of the batch against the numpy model: the
    id set of every query."""
    maps, trees, empty, reqs, b = scene
    batched(b, reqs)
    spec = SpecTree()
    spec.Build(maps[0].points)
    for r, want in ((reqs[1], spec.box_search(maps[0].boxes)),
                    (reqs[2], spec.radius_search(maps[0].radius_q, maps[0].radius))):
        off, ids, _ = r.outputs()
        assert len(want) == len(off) - 1
        for qi, w in enumerate(want):
            assert np.array_equal(np.sort(ids[off[qi]:off[qi + 1]]), np.asarray(w)), f"{r.kind} query {qi}"


def test_batch_after_mutation(ikdg_mod):
    maps, trees, empty, reqs, b = make_scene(ikdg_mod, 3202, 4, headroom=True)
    assert_same(batched(b, reqs), per_call(reqs), reqs)
    rng = np.random.default_rng(77)
    # pools grow (new device arrays) and boxes are deleted; the same graph runs
    for m, t in zip(maps, trees):
        lo, hi = m.points.min(0), m.points.max(0)
        t.Add_Points(rng.uniform(lo, hi, (len(m.points) // 2 + 1000, 3)).astype(np.float32), False)
        c = rng.uniform(lo, hi, (5, 3))
        t.Delete_Point_Boxes(np.concatenate([c - 4, c + 4], 1).astype(np.float32))
    empty.Add_Points(maps[0].points[:5000], False)
    ref = per_call(reqs)
    got = batched(b, reqs)
    assert_same(got, ref, reqs)
    # downsampled adds, then once more
    for t in trees:
        t.Add_Points(maps[0].points[:20000] + np.float32(0.25), True)
    ref = per_call(reqs)
    got = batched(b, reqs)
    assert_same(got, ref, reqs)
    b.close()


def test_batch_capacity_overflow(scene, ikdg_mod):
    maps, trees, empty, reqs, b = scene
    i = int(np.argmax([len(m.points) for m in maps]))
    # 10 m boxes centred on map points: every box holds points
    c = maps[i].points[:: max(1, len(maps[i].points) // 200)][:200]
    boxes = np.concatenate([c - 5, c + 5], 1).astype(np.float32)
    big = Req.rng("box", trees[i], boxes)
    tot = big.size_range()
    assert tot > 200
    small = Req.rng("box", trees[i], boxes, capacity=tot // 2)
    small.size_range()
    kn = Req.knn(trees[i], maps[i].knn_q, 5, math.inf)
    nb = ikdg_mod.Batch()
    small.add_to(nb)
    kn.add_to(nb)
    nb.run()
    with pytest.raises(ikdg_mod.IkdgError) as e:
        nb.synchronize(1)
    assert e.value.status == ikdg_mod.CAPACITY
    # the offsets and the kNN request are still complete
    off = small.offsets.cpu().numpy()
    assert off[-1] == tot
    ref = Req.knn(trees[i], maps[i].knn_q, 5, math.inf)
    assert_same([kn.outputs()], per_call([ref]), [kn])
    nb.close()


def test_autotune_keeps_results(scene):
    maps, trees, empty, reqs, b = scene
    before = batched(b, reqs)
    chosen = b.autotune(reps=2)
    assert chosen.shape[1] == 2 and len(chosen) == len(set(id(r.tree) for r in reqs))
    assert set(chosen[:, 0]) <= {8, 12, 16, 24, 32} and set(chosen[:, 1]) <= {1, 2, 4}
    after = batched(b, reqs)
    # the tuner rebuilt trees (new shapes): hits may come in another order
    assert_same_sets(after, before, reqs)
    assert_same(after, per_call(reqs), reqs)
    for t in trees:
        assert t.validate() == 0
