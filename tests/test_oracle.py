"""The oracle, pinned: the CPU restatement of the reference (oracle port) and
the brute-force numpy model both reproduce the golden fixtures that the
unmodified reference produced; where the reference itself is built here, the
port also matches it live on random operation sequences."""
import numpy as np
import pytest

import golden_check as G
import oracle_lib
import spec


@pytest.fixture(scope="module")
def port_lib():
    if not oracle_lib.available("port"):
        oracle_lib.build("port")
    return True


def port_tree(d, b, box):
    return G.Adapter(oracle_lib.OracleTree(d, b, box, kind="port"), "port")


def spec_tree(d, b, box):
    return G.Adapter(spec.SpecTree(box), "spec")


@pytest.mark.parametrize("replay", G.REPLAYS_TREE, ids=lambda f: f.__name__)
def test_port_reproduces_reference_fixtures(port_lib, replay):
    replay(port_tree)


@pytest.mark.parametrize("replay", G.REPLAYS, ids=lambda f: f.__name__)
def test_spec_reproduces_reference_fixtures(replay):
    replay(spec_tree)


def test_port_knn_order_identical_to_reference_fixture(port_lib):
    # Same algorithm and same build: the port returns the reference's rows in
    # the same order, bit for bit.
    g = G.load("knn")
    t = oracle_lib.OracleTree(0.5, 0.6, 0.2, kind="port")
    t.Build(g["pts"])
    xyz, d2, cnt = t.knn(g["q"], 5)
    assert np.array_equal(G.bits(xyz), G.bits(g["k5_xyz"]))
    assert np.array_equal(G.bits(d2), G.bits(g["k5_d2"]))
    assert np.array_equal(t.tree_range(), g["tree_range"])


@pytest.mark.skipif(not oracle_lib.available("ref"), reason="reference not built on this machine")
@pytest.mark.parametrize("seed", [0, 1])
def test_port_matches_reference_live(port_lib, seed):
    rng = np.random.default_rng(seed)
    L = 5.0
    pts = rng.uniform(-L, L, (3000, 3)).astype(np.float32)
    T = {k: oracle_lib.OracleTree(0.3, 0.6, 0.2, kind=k) for k in ("ref", "port")}
    for t in T.values():
        t.Build(pts)
    for it in range(10):
        add = rng.uniform(-L, L, (200, 3)).astype(np.float32)
        r = {k: t.Add_Points(add, bool(it % 2)) for k, t in T.items()}
        assert r["ref"] == r["port"]
        cur = T["port"].flatten()
        sel = cur[rng.choice(len(cur), 50, replace=False)]
        for t in T.values():
            t.Delete_Points(sel)
        c = rng.uniform(-L, L, (3, 3))
        s = rng.uniform(0.5, 3, (3, 3))
        b = np.concatenate([c - s / 2, c + s / 2], 1).astype(np.float32)
        assert T["ref"].Delete_Point_Boxes(b) == T["port"].Delete_Point_Boxes(b)
        if it % 5 == 4:
            for t in T.values():
                t.Add_Point_Boxes(b[:1])
        assert G.same_point_set(T["ref"].flatten(), T["port"].flatten())
        assert T["ref"].validnum() == T["port"].validnum()
        assert T["ref"].size() == T["port"].size()
        q = rng.uniform(-L, L, (200, 3)).astype(np.float32)
        a, b2 = T["ref"].knn(q, 5), T["port"].knn(q, 5)
        assert np.array_equal(G.bits(a[1]), G.bits(b2[1]))
        assert G.same_point_set(T["ref"].acquire_removed_points(), T["port"].acquire_removed_points())


def test_spec_knn_matches_port_distances(port_lib):
    rng = np.random.default_rng(5)
    pts = rng.uniform(-10, 10, (5000, 3)).astype(np.float32)
    q = rng.uniform(-10, 10, (300, 3)).astype(np.float32)
    p = oracle_lib.OracleTree(kind="port")
    p.Build(pts)
    s = spec.SpecTree()
    s.Build(pts)
    for k, md in ((5, np.inf), (12, 1.5)):
        xyz, d2, cnt = p.knn(q, k, md)
        ids, sd2 = s.knn(q, k, md)
        assert np.array_equal(cnt, (ids >= 0).sum(1))
        assert np.array_equal(G.bits(d2), G.bits(sd2))


@pytest.mark.skipif(not oracle_lib.available("ref"), reason="reference not built on this machine")
@pytest.mark.parametrize("kind", ["same", "plane", "lattice"])
def test_oracles_match_reference_on_tied_inputs(port_lib, kind):
    # The degenerate inputs of the GPU builder tests, small: every split key
    # ties.  Reference, port and model agree on kNN distances, box-search
    # sets, box-delete counts and the surviving points.
    rng = np.random.default_rng(31 + ["same", "plane", "lattice"].index(kind))
    n = 3000
    if kind == "same":
        pts = np.full((n, 3), 1.5, np.float32)
    elif kind == "plane":
        pts = rng.uniform(-10, 10, (n, 3)).astype(np.float32)
        pts[:, 2] = 0.0
    else:
        pts = rng.integers(-4, 4, (n, 3)).astype(np.float32)
    T = {k: oracle_lib.OracleTree(0.5, 0.6, 0.2, kind=k) for k in ("ref", "port")}
    s = spec.SpecTree()
    for t in T.values():
        t.Build(pts)
    s.Build(pts)
    q = (pts[rng.choice(n, 100)] + rng.normal(0, 0.7, (100, 3))).astype(np.float32)
    for k in (1, 5, 16):
        d2 = {name: t.knn(q, k)[1] for name, t in T.items()}
        _, sd2 = s.knn(q, k)
        assert np.array_equal(G.bits(d2["ref"]), G.bits(d2["port"]))
        assert np.array_equal(G.bits(d2["ref"]), G.bits(sd2))
    c = pts[rng.choice(n, 5)]
    h = rng.uniform(0.5, 3, (5, 3)).astype(np.float32)
    bx = np.concatenate([c - h, c + h], 1).astype(np.float32)
    (ro, rx), (po, px) = T["ref"].box_search(bx), T["port"].box_search(bx)
    want = s.box_search(bx)
    for i in range(len(bx)):
        assert G.same_point_set(rx[ro[i]:ro[i + 1]], px[po[i]:po[i + 1]])
        assert ro[i + 1] - ro[i] == len(want[i])
    nd = {name: t.Delete_Point_Boxes(bx[:2]) for name, t in T.items()}
    assert nd["ref"] == nd["port"] == s.Delete_Point_Boxes(bx[:2])
    assert T["ref"].validnum() == T["port"].validnum() == s.validnum()
    assert G.same_point_set(T["ref"].flatten(), T["port"].flatten())
    assert G.same_point_set(T["ref"].flatten(), s.valid_points()[0])
    for t in T.values():
        t.close()
