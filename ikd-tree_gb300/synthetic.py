"""Seeded synthetic inputs for the benchmark configurations.

No public dataset is involved: every workload is generated here from a seed, in
float32, with the shapes and distributions the configurations name.

* uniform maps / queries in a cube (the 1M-point kNN headline, the small plain
  case);
* a LiDAR-like world (ground plane z = 0 over 400 x 400 m plus vertical wall
  rectangles 2-30 m long and 3-15 m high at random yaw), a map sampled on its
  surfaces with 2 cm Gaussian noise, and rotating 32-beam scans (elevation
  -15..+15 deg, 625 azimuth steps, range 1-100 m) ray-cast against the same
  geometry along a 1 m/scan random walk;
* the sliding-window deletion of that workflow: the complement of a cube
  around the pose as at most six slab boxes;
* many independent maps with mixed kNN / box / radius query batches (the
  batched multi-map workload);
* a large map: uniform points in a flat slab plus planar clusters (the scale
  stress workload).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

F32 = np.float32
BIG = 1.0e9  # stands in for an unbounded slab side


def uniform(n: int, extent: float, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).uniform(-extent, extent, (n, 3)).astype(F32)


@dataclass
class World:
    half: float          # ground spans [-half, half]^2
    wall_c: np.ndarray   # [W, 2] wall centres
    wall_yaw: np.ndarray # [W]
    wall_len: np.ndarray # [W]
    wall_h: np.ndarray   # [W]


def lidar_world(seed: int, n_walls: int = 200, half: float = 200.0) -> World:
    rng = np.random.default_rng(seed)
    return World(half=half,
                 wall_c=rng.uniform(-half, half, (n_walls, 2)),
                 wall_yaw=rng.uniform(0, math.pi, n_walls),
                 wall_len=rng.uniform(2, 30, n_walls),
                 wall_h=rng.uniform(3, 15, n_walls))


def lidar_map(world: World, n: int, seed: int, noise: float = 0.02) -> np.ndarray:
    """n surface samples: ground and walls in proportion to their areas."""
    rng = np.random.default_rng(seed)
    ground_area = (2 * world.half) ** 2
    wall_area = world.wall_len * world.wall_h
    p_wall = wall_area / (ground_area + wall_area.sum())
    counts = rng.multinomial(n, np.concatenate([[1 - p_wall.sum()], p_wall]))
    g = np.c_[rng.uniform(-world.half, world.half, (counts[0], 2)), np.zeros(counts[0])]
    parts = [g]
    for i, m in enumerate(counts[1:]):
        if m == 0:
            continue
        s = rng.uniform(-world.wall_len[i] / 2, world.wall_len[i] / 2, m)
        h = rng.uniform(0, world.wall_h[i], m)
        c, yaw = world.wall_c[i], world.wall_yaw[i]
        parts.append(np.c_[c[0] + s * math.cos(yaw), c[1] + s * math.sin(yaw), h])
    p = np.concatenate(parts)
    p = p + rng.normal(0, noise, p.shape)
    return p[rng.permutation(len(p))].astype(F32)


def trajectory(n_scans: int, seed: int, step: float = 1.0):
    """Random walk in the plane, 1 m per scan, slowly turning heading."""
    rng = np.random.default_rng(seed)
    pos = np.zeros(2)
    yaw = rng.uniform(0, 2 * math.pi)
    poses = []
    for _ in range(n_scans):
        poses.append((pos[0], pos[1], yaw))
        yaw += rng.normal(0, 0.1)
        pos = pos + step * np.array([math.cos(yaw), math.sin(yaw)])
    return poses


def lidar_scan(world: World, pose, seed: int, beams: int = 32, azimuths: int = 625,
               height: float = 1.8, max_range: float = 100.0, noise: float = 0.02) -> np.ndarray:
    """Ray-casts a rotating multi-beam scan; returns the hit points (world frame)."""
    rng = np.random.default_rng(seed)
    px, py, yaw = pose
    elev = np.deg2rad(np.linspace(-15, 15, beams))
    az = yaw + np.linspace(0, 2 * math.pi, azimuths, endpoint=False)
    E, A = np.meshgrid(elev, az, indexing="ij")
    d = np.stack([np.cos(E) * np.cos(A), np.cos(E) * np.sin(A), np.sin(E)], -1).reshape(-1, 3)
    o = np.array([px, py, height])
    t = np.full(len(d), np.inf)
    down = d[:, 2] < 0
    t[down] = -o[2] / d[down, 2]
    gx = o[0] + t * d[:, 0]
    gy = o[1] + t * d[:, 1]
    t[(np.abs(gx) > world.half) | (np.abs(gy) > world.half)] = np.inf
    # walls: vertical rectangles, normal n = (-sin, cos, 0).  A wall whose
    # nearest point lies beyond max_range can only give hits that are dropped
    # below, so it is left out of the intersection (same output, less work).
    near = np.hypot(world.wall_c[:, 0] - o[0], world.wall_c[:, 1] - o[1]) - world.wall_len / 2 <= max_range
    wc, wyaw, wlen, wh = world.wall_c[near], world.wall_yaw[near], world.wall_len[near], world.wall_h[near]
    nx, ny = -np.sin(wyaw), np.cos(wyaw)
    ux, uy = np.cos(wyaw), np.sin(wyaw)
    denom = d[:, 0:1] * nx[None] + d[:, 1:2] * ny[None]                  # [R, W]
    num = (wc[:, 0] - o[0]) * nx + (wc[:, 1] - o[1]) * ny  # [W]
    with np.errstate(divide="ignore", invalid="ignore"):
        tw = num[None] / denom
    hx = o[0] + tw * d[:, 0:1]
    hy = o[1] + tw * d[:, 1:2]
    hz = o[2] + tw * d[:, 2:3]
    along = (hx - wc[:, 0]) * ux + (hy - wc[:, 1]) * uy
    ok = (tw > 0) & (np.abs(along) <= wlen / 2) & (hz >= 0) & (hz <= wh)
    tw = np.where(ok, tw, np.inf).min(1)
    t = np.minimum(t, tw)
    keep = (t >= 1.0) & (t <= max_range)
    r = t[keep] + rng.normal(0, noise, keep.sum())
    return (o + r[:, None] * d[keep]).astype(F32)


def cube_complement_boxes(center, half: float) -> np.ndarray:
    """Boxes covering everything outside the cube center +- half (<= 6 slabs)."""
    cx, cy, cz = center
    lo = np.array([cx - half, cy - half, cz - half], F32)
    hi = np.array([cx + half, cy + half, cz + half], F32)
    b = []
    b.append([-BIG, -BIG, -BIG, lo[0], BIG, BIG])           # x < lo
    b.append([hi[0], -BIG, -BIG, BIG, BIG, BIG])            # x >= hi
    b.append([lo[0], -BIG, -BIG, hi[0], lo[1], BIG])        # y < lo
    b.append([lo[0], hi[1], -BIG, hi[0], BIG, BIG])         # y >= hi
    b.append([lo[0], lo[1], -BIG, hi[0], hi[1], lo[2]])     # z < lo
    b.append([lo[0], lo[1], hi[2], hi[0], hi[1], BIG])      # z >= hi
    return np.asarray(b, F32)


@dataclass
class MapRequests:
    """One map of the multi-map workload and its three query batches."""
    points: np.ndarray     # [N, 3]
    knn_q: np.ndarray      # [nk, 3]
    k: int
    max_dist: float
    boxes: np.ndarray      # [nb, 6] {min xyz, max xyz}
    radius_q: np.ndarray   # [nr, 3]
    radius: np.ndarray     # [nr]


def multi_maps(seed: int, n_maps: int = 64, size_range=(1e4, 1e6), query_range=(1e3, 1e5),
               side_range=(20.0, 200.0), kmax: int = 16) -> list[MapRequests]:
    """Independent maps with sizes log-uniform in size_range, each uniform in
    its own AABB (sides uniform in side_range); per map a query batch of
    log-uniform size split 60 % kNN (k uniform in 1..kmax, max_dist uniform in
    1-10 m), 20 % cubic boxes (side uniform in 0.5-5 m), 20 % radius queries
    (r uniform in 0.5-5 m), all centred uniformly in the map's AABB."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_maps):
        n = int(round(math.exp(rng.uniform(math.log(size_range[0]), math.log(size_range[1])))))
        sides = rng.uniform(side_range[0], side_range[1], 3)
        lo = rng.uniform(-500.0, 500.0, 3)
        pts = (lo + rng.uniform(0.0, 1.0, (n, 3)) * sides).astype(F32)
        nq = int(round(math.exp(rng.uniform(math.log(query_range[0]), math.log(query_range[1])))))
        nk = int(round(0.6 * nq))
        nb = int(round(0.2 * nq))
        nr = nq - nk - nb

        def centres(m):
            return (lo + rng.uniform(0.0, 1.0, (m, 3)) * sides).astype(F32)

        kq = centres(nk)
        k = int(rng.integers(1, kmax + 1))
        max_dist = float(rng.uniform(1.0, 10.0))
        bc = centres(nb)
        half = (rng.uniform(0.5, 5.0, nb) / 2.0).astype(F32)[:, None]
        boxes = np.concatenate([bc - half, bc + half], axis=1).astype(F32)
        rq = centres(nr)
        rad = rng.uniform(0.5, 5.0, nr).astype(F32)
        out.append(MapRequests(pts, kq, k, max_dist, boxes, rq, rad))
    return out


def stress_map(n: int, seed: int, n_clusters: int = 400, cluster_frac: float = 0.3) -> np.ndarray:
    """Uniform points in [-500, 500]^2 x [0, 50] m plus planar clusters: a
    fraction of the points lies on random planar patches (10-60 m wide
    rectangles at random orientation, 2 cm noise)."""
    rng = np.random.default_rng(seed)
    nc = int(n * cluster_frac)
    nu = n - nc
    u = np.empty((nu, 3), F32)
    u[:, 0:2] = rng.uniform(-500.0, 500.0, (nu, 2))
    u[:, 2] = rng.uniform(0.0, 50.0, nu)
    which = rng.integers(0, n_clusters, nc)
    centre = np.stack([rng.uniform(-500, 500, n_clusters), rng.uniform(-500, 500, n_clusters),
                       rng.uniform(0, 50, n_clusters)], 1)
    normal = rng.normal(size=(n_clusters, 3))
    normal /= np.linalg.norm(normal, axis=1, keepdims=True)
    a = np.cross(normal, np.array([0.0, 0.0, 1.0]))
    bad = np.linalg.norm(a, axis=1) < 1e-6
    a[bad] = np.cross(normal[bad], np.array([1.0, 0.0, 0.0]))
    a /= np.linalg.norm(a, axis=1, keepdims=True)
    b = np.cross(normal, a)
    w = rng.uniform(10.0, 60.0, (n_clusters, 2))
    s = rng.uniform(-0.5, 0.5, (nc, 2)) * w[which]
    c = (centre[which] + s[:, :1] * a[which] + s[:, 1:] * b[which] +
         rng.normal(0.0, 0.02, (nc, 1)) * normal[which])
    return np.concatenate([u, c.astype(F32)])[rng.permutation(n)].astype(F32)


def random_boxes(m: int, seed: int, side_range=(1.0, 20.0), lo=(-500.0, -500.0, 0.0),
                 hi=(500.0, 500.0, 50.0)) -> np.ndarray:
    """m axis-aligned boxes, centres uniform in [lo, hi], sides uniform in
    side_range per axis."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(lo, hi, (m, 3))
    h = rng.uniform(side_range[0], side_range[1], (m, 3)) / 2.0
    return np.concatenate([c - h, c + h], axis=1).astype(F32)
