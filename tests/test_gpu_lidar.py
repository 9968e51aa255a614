"""LiDAR-like incremental mapping at full size, GPU against the oracle port.

A 2M-point map (ground plane plus 200 walls, 2 cm noise) and a stream of
ray-cast 32-beam scans along a 1 m/scan random walk.  Per scan, exactly as a
mapping front end does: kNN (k = 5, max_dist = 5 m) for every scan point,
Add_Points with 0.5 m voxel downsampling, and Delete_Point_Boxes keeping a
200 m cube around the pose.  Every return value, every squared distance, the
neighbour sets and the full set of valid points must match the CPU
restatement of the reference.
"""
import numpy as np
import pytest

import golden_check as G
import oracle_lib
import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def port_ready():
    if not oracle_lib.available("port"):
        oracle_lib.build("port")


def test_lidar_stream_matches_port(ikdg_mod, port_ready):
    world = S.lidar_world(2001)
    base = S.lidar_map(world, 2_000_000, 2002)
    poses = S.trajectory(10, 2003)
    gpu = ikdg_mod.KDTree(0.5, 0.6, 0.5)
    cpu = oracle_lib.OracleTree(0.5, 0.6, 0.5, kind="port")
    gpu.Build(base)
    cpu.Build(base)
    for s, pose in enumerate(poses):
        scan = S.lidar_scan(world, pose, 5000 + s)
        ids, d2, xyz, cnt = gpu.knn(scan, 5, 5.0)
        rxyz, rd2, rcnt = cpu.knn(scan, 5, 5.0, nthreads=8)
        G.check_knn_rows(scan, rxyz, rd2, rcnt, xyz, d2, cnt)
        assert gpu.Add_Points(scan, True) == cpu.Add_Points(scan, True), f"scan {s}: downsampled inserts"
        boxes = S.cube_complement_boxes((pose[0], pose[1], 1.8), 100.0)
        assert gpu.Delete_Point_Boxes(boxes) == cpu.Delete_Point_Boxes(boxes), f"scan {s}: deleted count"
        assert gpu.validnum() == cpu.validnum(), f"scan {s}: validnum"
        if s in (0, len(poses) - 1):
            assert G.same_point_set(gpu.flatten(), cpu.flatten()), f"scan {s}: valid point sets differ"


def test_lidar_hundred_scans(ikdg_mod, port_ready):
    """The whole stream of the LiDAR configuration: 100 scans.  Every scan's
    downsampled-insert and deleted counts equal the port's, the structure
    validates at the end, and the final valid point sets are identical; the
    neighbours are compared on every tenth scan."""
    world = S.lidar_world(2101)
    base = S.lidar_map(world, 2_000_000, 2102)
    poses = S.trajectory(100, 2103)
    gpu = ikdg_mod.KDTree(0.5, 0.6, 0.5)
    cpu = oracle_lib.OracleTree(0.5, 0.6, 0.5, kind="port")
    gpu.Build(base)
    cpu.Build(base)
    for s, pose in enumerate(poses):
        scan = S.lidar_scan(world, pose, 6000 + s)
        if s % 10 == 0:
            ids, d2, xyz, cnt = gpu.knn(scan, 5, 5.0)
            rxyz, rd2, rcnt = cpu.knn(scan, 5, 5.0, nthreads=8)
            G.check_knn_rows(scan, rxyz, rd2, rcnt, xyz, d2, cnt)
        assert gpu.Add_Points(scan, True) == cpu.Add_Points(scan, True), f"scan {s}: downsampled inserts"
        boxes = S.cube_complement_boxes((pose[0], pose[1], 1.8), 100.0)
        assert gpu.Delete_Point_Boxes(boxes) == cpu.Delete_Point_Boxes(boxes), f"scan {s}: deleted count"
    assert gpu.validnum() == cpu.validnum()
    assert gpu.validate() == 0
    assert G.same_point_set(gpu.flatten(), cpu.flatten()), "valid point sets differ after 100 scans"
