"""The seeded workload generators (CPU): determinism, shapes, ranges and the
distributions the configurations name."""
import math

import numpy as np

import synthetic as S


def test_multi_maps_shapes_and_ranges():
    a = S.multi_maps(11, n_maps=6, size_range=(1e3, 1e4), query_range=(100, 1000))
    b = S.multi_maps(11, n_maps=6, size_range=(1e3, 1e4), query_range=(100, 1000))
    assert len(a) == 6
    for m, m2 in zip(a, b):
        assert np.array_equal(m.points, m2.points) and m.k == m2.k and m.max_dist == m2.max_dist
        assert m.points.dtype == np.float32 and m.points.shape[1] == 3
        assert 1e3 - 1 <= len(m.points) <= 1e4 + 1
        ext = m.points.max(0) - m.points.min(0)
        assert np.all(ext <= 200.0) and np.all(ext >= 10.0)
        nq = len(m.knn_q) + len(m.boxes) + len(m.radius_q)
        assert 100 <= nq <= 1001
        assert abs(len(m.knn_q) - 0.6 * nq) <= 1 and abs(len(m.boxes) - 0.2 * nq) <= 1
        assert 1 <= m.k <= 16 and 1.0 <= m.max_dist <= 10.0
        side = m.boxes[:, 3:] - m.boxes[:, :3]
        assert np.all(side >= 0.5 - 1e-3) and np.all(side <= 5.0 + 1e-3)
        assert np.allclose(side[:, 0], side[:, 1], atol=1e-3) and np.allclose(side[:, 0], side[:, 2], atol=1e-3)
        assert np.all(m.radius >= 0.5) and np.all(m.radius <= 5.0)
        lo, hi = m.points.min(0) - 1e-3, m.points.max(0) + 1e-3
        assert np.all((m.knn_q >= lo - 5) & (m.knn_q <= hi + 5))


def test_stress_map_and_boxes():
    p = S.stress_map(200_000, 3, n_clusters=20)
    assert p.shape == (200_000, 3) and p.dtype == np.float32
    assert np.all(np.abs(p[:, :2]) <= 560) and p[:, 2].min() > -40 and p[:, 2].max() < 90
    assert np.array_equal(p, S.stress_map(200_000, 3, n_clusters=20))
    b = S.random_boxes(100, 4)
    side = b[:, 3:] - b[:, :3]
    assert b.shape == (100, 6) and np.all(side >= 1.0 - 1e-4) and np.all(side <= 20.0 + 1e-4)


def test_lidar_scan_geometry():
    w = S.lidar_world(5, n_walls=20)
    pose = S.trajectory(1, 6)[0]
    s = S.lidar_scan(w, pose, 7)
    assert s.dtype == np.float32 and s.shape[1] == 3 and 0 < len(s) <= 32 * 625
    r = np.linalg.norm(s[:, :2] - np.asarray(pose[:2], np.float32), axis=1)
    assert r.max() <= 100.0 + 1.0
    boxes = S.cube_complement_boxes((pose[0], pose[1], 1.8), 100.0)
    assert boxes.shape[1] == 6 and len(boxes) <= 6
