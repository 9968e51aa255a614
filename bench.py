#!/usr/bin/env python
"""Benchmark: batched kNN (k=5) on a 1M-point map, 100k-query batches.

One step = one batch of 100k Nearest_Search queries (k = 5, max_dist = inf)
against a 1M-point map (uniform in [-50, 50]^3, float32, seeded synthetic data).

  value  - queries/s with the queries already in HBM (ikdg_knn_device), timed
           with CUDA events on the tree's stream; L2 is flushed (512 MB write)
           before every timed step, outside the events.
  e2e    - the same metric through the host C ABI (ikdg_knn): host queries in,
           ids + squared distances + points out, copies included.
  roofline - the kNN kernel against the measured HBM copy bandwidth, with the
           algorithmic bytes per query 12 + 8k + 16*32 + 32*ceil(log2(N/32)).
  update_ms_per_scan - LiDAR-like incremental mapping: a 2M-point map (ground
           plane + 200 walls), ray-cast 32x625 scans along a 1 m/scan walk;
           per scan Add_Points with 0.5 m voxel downsampling plus
           Delete_Point_Boxes keeping a 200 m cube around the pose, through
           the host API (median over the scans after the first; the first
           scan's deletion removes most of the map and is reported apart).
  cpu_baseline - the CPU restatement of the reference (oracle port) on this
           host's cores, same map and queries.
  stress - a 20M-point map (uniform slab plus planar clusters): device kNN of
           1M queries at k in {1, 5, 16, 32} (max 2 m) with the achieved
           fraction of the HBM roofline, radius search r = 1 m, 1000 box
           deletions (1-20 m sides), then the same queries again.
  batched - 64 independent maps (10k-1M points each, 14.7M in all) with
           log-uniform query batches (1.37M queries: 60 % kNN k 1-16, 20 %
           box, 20 % radius), all on device buffers: the plain per-call
           device path (one ikdg_*_device call per request) against one
           graph launch of a multi-tree batch, host wall clock around issue
           and completion of each, before and after the batch autotuner.

`--impl reference` times that CPU implementation alone on the same workload.
Multi-GPU (torchrun): every rank holds its own replica of the tree (the path
does not shard); value is the sum over ranks, timing is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "ikd-tree_gb300")
ORACLE = os.path.join(ROOT, "oracle")
sys.path.insert(0, PKG)

N_MAP = 1_000_000
N_Q = 100_000
K = 5
EXTENT = 50.0
MAP_SEED = 1002
DS = 0.5
WORKLOAD = "knn_k5_map1M_uniform_q100k"
METRIC = "kNN queries/sec (k=5, 1M map)"


def bytes_per_query(n: int, k: int) -> int:
    depth = math.ceil(math.log2(n / 32))
    return 12 + 8 * k + 16 * 32 + 32 * depth


def make_map() -> np.ndarray:
    return np.random.default_rng(MAP_SEED).uniform(-EXTENT, EXTENT, (N_MAP, 3)).astype(np.float32)


def make_queries(step: int) -> np.ndarray:
    return np.random.default_rng(7000 + step).uniform(-EXTENT, EXTENT, (N_Q, 3)).astype(np.float32)


LIDAR_MAP = 2_000_000
LIDAR_SCANS = 100
_LIDAR = None


def lidar_workload():
    """The LiDAR-like mapping stream: base map, then per scan (points, boxes).
    Generated once per process (ray casting 100 scans takes a few seconds)."""
    global _LIDAR
    if _LIDAR is None:
        import synthetic as S
        world = S.lidar_world(2001)
        base = S.lidar_map(world, LIDAR_MAP, 2002)
        scans = []
        for s, pose in enumerate(S.trajectory(LIDAR_SCANS, 2003)):
            pts = S.lidar_scan(world, pose, 5000 + s)
            scans.append((pts, S.cube_complement_boxes((pose[0], pose[1], 1.8), 100.0)))
        _LIDAR = (base, scans)
    return _LIDAR


def run_scans(tree, scans, knn):
    """Per scan: kNN of the scan (k=5, 5 m), then the timed map update."""
    knn_ms, upd_ms = [], []
    for pts, boxes in scans:
        t0 = time.perf_counter()
        knn(pts)
        t1 = time.perf_counter()
        tree.Add_Points(pts, True)
        tree.Delete_Point_Boxes(boxes)
        t2 = time.perf_counter()
        knn_ms.append(1e3 * (t1 - t0))
        upd_ms.append(1e3 * (t2 - t1))
    return {"update_ms_per_scan": statistics.median(upd_ms[1:]), "update_ms_first_scan": upd_ms[0],
            "scan_knn_ms": statistics.median(knn_ms[1:]),
            "scan_points": int(statistics.median([len(p) for p, _ in scans]))}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def knn_traffic():
    """Per-launch DRAM bytes of the kNN kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "knn_traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f).get("dram_bytes_per_launch")
    return None


class ClockSampler:
    def __init__(self, device: int):
        self.path = tempfile.mktemp(suffix=".csv")
        fields = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                  "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                  "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={fields}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


MM_SEED = 3001
STRESS_N = 20_000_000
STRESS_Q = 1_000_000


def range_bench(tree, torch, dev, reps: int = 3) -> dict:
    """Box and radius search of RANGE_Q queries each on the headline map
    through the device entry points (count pass, prefix sum, write pass),
    CUDA events on the tree stream, median of `reps`."""
    boxes, centres, radius = range_queries()
    st = torch.cuda.ExternalStream(tree.stream(), device=dev)
    b = torch.from_numpy(boxes).to(dev)
    c = torch.from_numpy(centres).to(dev)
    r = torch.from_numpy(radius).to(dev)
    offs = torch.empty((RANGE_Q + 1,), dtype=torch.int64, device=dev)
    total = torch.zeros((1,), dtype=torch.int64, device=dev)
    out = {"workload": f"{RANGE_Q} boxes (side U(0.5,5) m per axis) and {RANGE_Q} radius queries "
                       "(r U(0.5,5) m) on the 1M-point uniform map; ids and points out",
           "timing": f"CUDA events on the tree stream, median of {reps}"}
    for name, call in (("box", lambda i, cap, x: tree.box_search_device(b.data_ptr(), RANGE_Q, offs.data_ptr(), i,
                                                                         cap, x, total.data_ptr())),
                       ("radius", lambda i, cap, x: tree.radius_search_device(c.data_ptr(), RANGE_Q, r.data_ptr(),
                                                                               offs.data_ptr(), i, cap, x,
                                                                               total.data_ptr()))):
        call(0, 0, 0)
        tree.synchronize()
        cap = int(total.item())
        rid = torch.empty((max(cap, 1),), dtype=torch.int32, device=dev)
        rxyz = torch.empty((max(cap, 1), 3), dtype=torch.float32, device=dev)
        call(rid.data_ptr(), cap, rxyz.data_ptr())
        tree.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            call(rid.data_ptr(), cap, rxyz.data_ptr())
            e1.record(st)
            tree.synchronize()
            ts.append(e0.elapsed_time(e1))
        ms = statistics.median(ts)
        out[f"{name}_ms"] = ms
        out[f"{name}_queries_per_s"] = RANGE_Q / (ms / 1e3)
        out[f"{name}_hits"] = cap
    return out


def facade_bench(threads: int = 8) -> dict:
    """Per-point Nearest_Search through the C++ drop-in facade: the call
    shape of a front end that searches point by point, on one thread and on
    `threads` threads (ikd-tree_gb300/facade_latency.cpp)."""
    exe = os.path.join(tempfile.mkdtemp(), "facade_latency")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(PKG, "facade_latency.cpp"), "-o", exe, "-L", PKG, "-likdg", f"-Wl,-rpath,{PKG}",
           "-L/usr/local/cuda/lib64", "-lcudart", "-pthread"]
    try:
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        r = subprocess.run([exe, str(N_MAP), "20000", str(threads)], check=True, capture_output=True, text=True,
                           timeout=600)
        return json.loads(r.stdout.strip().splitlines()[-1])
    except (subprocess.SubprocessError, OSError, ValueError) as e:
        return {"error": str(e)[:300]}


def stress_bench(ikdg, torch, device: int, reps: int = 3) -> dict:
    """Scale stress: 20M-point map, 1M-query batches, 1000 box deletions."""
    import synthetic as S
    dev = torch.device("cuda", device)
    pts = S.stress_map(STRESS_N, 5005)
    rng = np.random.default_rng(5006)
    qh = np.empty((STRESS_Q, 3), np.float32)
    qh[:, :2] = rng.uniform(-500, 500, (STRESS_Q, 2))
    qh[:, 2] = rng.uniform(0, 50, STRESS_Q)
    tree = ikdg.KDTree(0.5, 0.6, DS, device=device)
    t0 = time.perf_counter()
    tree.Build(pts)
    build_ms = 1e3 * (time.perf_counter() - t0)
    st = torch.cuda.ExternalStream(tree.stream(), device=dev)
    q = torch.from_numpy(qh).to(dev)
    kmax = 32
    ids = torch.empty((STRESS_Q, kmax), dtype=torch.int32, device=dev)
    d2 = torch.empty((STRESS_Q, kmax), dtype=torch.float32, device=dev)
    xyz = torch.empty((STRESS_Q, kmax, 3), dtype=torch.float32, device=dev)
    cnt = torch.empty((STRESS_Q,), dtype=torch.int32, device=dev)
    offs = torch.empty((STRESS_Q + 1,), dtype=torch.int64, device=dev)
    total = torch.zeros((1,), dtype=torch.int64, device=dev)
    radius = torch.full((STRESS_Q,), 1.0, dtype=torch.float32, device=dev)
    peak, _ = measured_peak()

    def ev_time(fn):
        fn()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            tree.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    def queries():
        out = {}
        for k in (1, 5, 16, 32):
            ms = ev_time(lambda: tree.knn_device(q.data_ptr(), STRESS_Q, k, 2.0, ids.data_ptr(), d2.data_ptr(),
                                                 xyz.data_ptr(), cnt.data_ptr()))
            gbs = STRESS_Q * bytes_per_query(tree.validnum(), k) / (ms / 1e3) / 1e9
            out[f"knn_k{k}"] = {"ms": ms, "queries_per_s": STRESS_Q / (ms / 1e3), "achieved_gbs": gbs,
                                "hbm_frac": gbs / peak,
                                "mean_count": float(cnt.float().mean().item())}
        tree.radius_search_device(q.data_ptr(), STRESS_Q, radius.data_ptr(), offs.data_ptr(), 0, 0, 0,
                                  total.data_ptr())
        tree.synchronize()
        cap = int(total.item())
        rid = torch.empty((max(cap, 1),), dtype=torch.int32, device=dev)
        rxyz = torch.empty((max(cap, 1), 3), dtype=torch.float32, device=dev)
        ms = ev_time(lambda: tree.radius_search_device(q.data_ptr(), STRESS_Q, radius.data_ptr(), offs.data_ptr(),
                                                       rid.data_ptr(), cap, rxyz.data_ptr(), total.data_ptr()))
        out["radius_r1"] = {"ms": ms, "queries_per_s": STRESS_Q / (ms / 1e3), "hits": cap}
        return out

    before = queries()
    boxes = S.random_boxes(1000, 5007)
    t0 = time.perf_counter()
    n_del = tree.Delete_Point_Boxes(boxes)
    del_ms = 1e3 * (time.perf_counter() - t0)
    after = queries()
    res = {"workload": f"{STRESS_N} points (uniform slab [-500,500]^2 x [0,50] m + planar clusters), "
                       f"{STRESS_Q} uniform queries, k in 1/5/16/32 max 2 m, radius 1 m, 1000 boxes 1-20 m",
           "build_ms": build_ms, "before": before, "delete_1000_boxes_ms": del_ms, "deleted": n_del,
           "after": after, "timing": f"CUDA events on the tree stream, median of {reps}; inputs > L2"}
    tree.close()
    return res


def multimap_bench(ikdg, torch, device: int, reps: int = 5, tune: bool = True) -> dict:
    """Plain per-call device path vs one graph launch of a multi-tree batch."""
    import synthetic as S
    dev = torch.device("cuda", device)
    maps = S.multi_maps(MM_SEED)
    trees, reqs = [], []
    for m in maps:
        t = ikdg.KDTree(0.5, 0.6, DS, device=device)
        t.Build(m.points)
        trees.append(t)

    def zeros(shape, dt):
        return torch.empty(shape, dtype=dt, device=dev)

    n_queries = 0
    for m, t in zip(maps, trees):
        nk, nb, nr = len(m.knn_q), len(m.boxes), len(m.radius_q)
        n_queries += nk + nb + nr
        reqs.append(("knn", t, dict(q=torch.from_numpy(m.knn_q).to(dev), nq=nk, k=m.k, md=m.max_dist,
                                    ids=zeros((nk, m.k), torch.int32), d2=zeros((nk, m.k), torch.float32),
                                    xyz=zeros((nk, m.k, 3), torch.float32), cnt=zeros((nk,), torch.int32))))
        for kind, q, n, rad in (("box", m.boxes, nb, None), ("radius", m.radius_q, nr, m.radius)):
            r = dict(q=torch.from_numpy(q).to(dev), nq=n, offs=zeros((n + 1,), torch.int64),
                     total=torch.zeros((1,), dtype=torch.int64, device=dev),
                     rad=torch.from_numpy(rad).to(dev) if rad is not None else None)
            if kind == "box":
                t.box_search_device(r["q"].data_ptr(), n, r["offs"].data_ptr(), 0, 0, 0, r["total"].data_ptr())
            else:
                t.radius_search_device(r["q"].data_ptr(), n, r["rad"].data_ptr(), r["offs"].data_ptr(), 0, 0, 0,
                                       r["total"].data_ptr())
            t.synchronize()
            cap = int(r["total"].item())
            r["cap"] = cap
            r["ids"] = zeros((max(cap, 1),), torch.int32)
            r["xyz"] = zeros((max(cap, 1), 3), torch.float32)
            reqs.append((kind, t, r))
    n_hits = sum(r["cap"] for kind, _, r in reqs if kind != "knn")
    n_range = sum(1 for kind, _, _ in reqs if kind != "knn")

    def plain():
        for kind, t, r in reqs:
            if kind == "knn":
                t.knn_device(r["q"].data_ptr(), r["nq"], r["k"], r["md"], r["ids"].data_ptr(), r["d2"].data_ptr(),
                             r["xyz"].data_ptr(), r["cnt"].data_ptr())
            elif kind == "box":
                t.box_search_device(r["q"].data_ptr(), r["nq"], r["offs"].data_ptr(), r["ids"].data_ptr(),
                                    r["cap"], r["xyz"].data_ptr(), r["total"].data_ptr())
            else:
                t.radius_search_device(r["q"].data_ptr(), r["nq"], r["rad"].data_ptr(), r["offs"].data_ptr(),
                                       r["ids"].data_ptr(), r["cap"], r["xyz"].data_ptr(), r["total"].data_ptr())
        for t in trees:
            t.synchronize()

    def plain_sync():
        # each request awaited before the next, as a caller consuming every
        # result in turn (the reference's calls are synchronous)
        for kind, t, r in reqs:
            if kind == "knn":
                t.knn_device(r["q"].data_ptr(), r["nq"], r["k"], r["md"], r["ids"].data_ptr(), r["d2"].data_ptr(),
                             r["xyz"].data_ptr(), r["cnt"].data_ptr())
            elif kind == "box":
                t.box_search_device(r["q"].data_ptr(), r["nq"], r["offs"].data_ptr(), r["ids"].data_ptr(),
                                    r["cap"], r["xyz"].data_ptr(), r["total"].data_ptr())
            else:
                t.radius_search_device(r["q"].data_ptr(), r["nq"], r["rad"].data_ptr(), r["offs"].data_ptr(),
                                       r["ids"].data_ptr(), r["cap"], r["xyz"].data_ptr(), r["total"].data_ptr())
            t.synchronize()

    b = ikdg.Batch(device)
    for kind, t, r in reqs:
        if kind == "knn":
            b.add_knn(t, r["q"].data_ptr(), r["nq"], r["k"], r["md"], r["ids"].data_ptr(), r["d2"].data_ptr(),
                      r["xyz"].data_ptr(), r["cnt"].data_ptr())
        elif kind == "box":
            b.add_box_search(t, r["q"].data_ptr(), r["nq"], r["offs"].data_ptr(), r["ids"].data_ptr(), r["cap"],
                             r["xyz"].data_ptr())
        else:
            b.add_radius_search(t, r["q"].data_ptr(), r["nq"], r["rad"].data_ptr(), r["offs"].data_ptr(),
                                r["ids"].data_ptr(), r["cap"], r["xyz"].data_ptr())

    def batched():
        b.run()
        b.synchronize(n_range)

    def timed(fn):
        fn()
        fn()
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            ts.append(1e3 * (time.perf_counter() - t0))
        return statistics.median(ts)

    def batch_device_ms():
        st = torch.cuda.ExternalStream(b.stream, device=dev)
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            b.run()
            e1.record(st)
            b.synchronize(n_range)
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    plain_ms = timed(plain)
    plain_sync_ms = timed(plain_sync)
    b.set_query_order(True)
    batch_ordered_ms = timed(batched)
    b.set_query_order(False)

    batch_ms = timed(batched)
    batch_dev = batch_device_ms()
    tuned = None
    if tune:
        t0 = time.perf_counter()
        chosen = b.autotune(3)
        tune_s = time.perf_counter() - t0
        tuned_ms = timed(batched)
        tuned_dev = batch_device_ms()
        plain_tuned_ms = timed(plain)
        tuned = {"batched_ms": tuned_ms, "batched_device_ms": tuned_dev, "plain_ms": plain_tuned_ms,
                 "speedup_vs_plain": plain_tuned_ms / tuned_ms, "tune_s": tune_s,
                 "fill_counts": {str(f): int((chosen[:, 0] == f).sum()) for f in sorted(set(chosen[:, 0]))},
                 "lanes_counts": {str(l): int((chosen[:, 1] == l).sum()) for l in sorted(set(chosen[:, 1]))}}
    out = {
        "workload": f"{len(maps)} maps, {sum(len(m.points) for m in maps)} points, {n_queries} queries "
                    f"(60% kNN k 1-16 max 1-10 m, 20% box 0.5-5 m, 20% radius 0.5-5 m), {n_hits} range hits, "
                    "ids + points out; inputs larger than L2",
        "queries": n_queries,
        "plain_ms": plain_ms, "plain_queries_per_s": n_queries / (plain_ms / 1e3),
        "plain": "per-call device entry points, asynchronous, each tree on its own stream (requests of "
                 "different trees overlap); one wait at the end",
        "plain_sync_ms": plain_sync_ms,
        "plain_sync": "the same calls, each awaited before the next",
        "batched_ms": batch_ms, "batched_queries_per_s": n_queries / (batch_ms / 1e3),
        "batched_device_ms": batch_dev,
        "batched_ordered_ms": batch_ordered_ms,
        "batched_ordered": "the same batch with every kNN request's queries sorted by a Morton code first",
        "speedup_vs_plain": plain_ms / batch_ms,
        "speedup_vs_plain_sync": plain_sync_ms / batch_ms,
        "autotuned": tuned,
        "plain_launches": 64 + n_range * 5,
        "timing": "host wall clock from issue to completion, median of %d runs" % reps,
    }
    b.close()
    for t in trees:
        t.close()
    return out


CONFIG = {"workload": WORKLOAD, "map_points": N_MAP, "queries_per_step": N_Q, "k": K, "max_dist": "inf",
          "l2": "GPU arm: flushed before every timed step by a 512 MB write (host arm: no flush)"}
PARITY_SAMPLE = 2000
RANGE_Q = 100_000


def range_queries():
    """Box (side U(0.5, 5) m per axis) and radius (r U(0.5, 5) m) queries
    centred uniformly in the headline map's cube: the range-search sizes of
    the batched multi-map workload, on the 1M-point map."""
    rng = np.random.default_rng(7500)
    c = rng.uniform(-EXTENT, EXTENT, (RANGE_Q, 3))
    side = rng.uniform(0.5, 5.0, (RANGE_Q, 3))
    boxes = np.concatenate([c - side / 2, c + side / 2], 1).astype(np.float32)
    centres = rng.uniform(-EXTENT, EXTENT, (RANGE_Q, 3)).astype(np.float32)
    radius = rng.uniform(0.5, 5.0, RANGE_Q).astype(np.float32)
    return boxes, centres, radius


def oracle_kind():
    """The CPU implementation timed beside the GPU: the unmodified reference
    (oracle/_ref/libikd_ref.so, compiled from the reference install in
    baseline/_ref/) when it is there, else the oracle port."""
    if ORACLE not in sys.path:
        sys.path.insert(0, ORACLE)
    import oracle_lib
    if not oracle_lib.available("ref") and os.path.isfile(
            os.path.join(ROOT, "baseline", "_ref", "ikd-Tree", "ikd_Tree.cpp")):
        try:
            oracle_lib.build("ref")
        except Exception:
            pass
    if oracle_lib.available("ref"):
        return "ref"
    if not oracle_lib.available("port"):
        oracle_lib.build("port")
    return "port"


KIND_NAME = {"ref": "reference", "port": "port"}


class StdoutToStderr:
    """Sends what native code prints to stdout (the reference announces its
    rebuild thread with printf) to stderr, so stdout carries only the JSON
    line."""

    def __enter__(self):
        sys.stdout.flush()
        self.saved = os.dup(1)
        os.dup2(2, 1)
        return self

    def __exit__(self, *exc):
        sys.stdout.flush()
        import ctypes
        ctypes.CDLL(None).fflush(None)  # C stdio buffers, still on stderr's descriptor
        os.dup2(self.saved, 1)
        os.close(self.saved)


def knn_rows_match(q, ref_xyz, ref_d2, ref_cnt, got_xyz, got_d2, got_cnt) -> int:
    """Rows whose kNN result differs (counts, squared-distance bits, and the
    neighbour points where no two distances of the row tie; tied rows accept
    any point at the tied distance)."""
    bad = 0
    ref_d2 = np.asarray(ref_d2, np.float32)
    got_d2 = np.asarray(got_d2, np.float32)
    for i in range(len(q)):
        c = int(ref_cnt[i])
        if int(got_cnt[i]) != c:
            bad += 1
            continue
        rd, gd = ref_d2[i, :c].view(np.uint32), got_d2[i, :c].view(np.uint32)
        if not np.array_equal(rd, gd):
            bad += 1
            continue
        if len(np.unique(rd)) == c:
            if not np.array_equal(np.asarray(ref_xyz[i, :c], np.float32).view(np.uint32),
                                  np.asarray(got_xyz[i, :c], np.float32).view(np.uint32)):
                bad += 1
            continue
        for j in range(c):
            p = np.asarray(got_xyz[i, j], np.float32)
            d = (q[i][0] - p[0]) * (q[i][0] - p[0]) + (q[i][1] - p[1]) * (q[i][1] - p[1])
            d = np.float32(np.float32(d) + np.float32((q[i][2] - p[2]) * (q[i][2] - p[2])))
            if np.float32(d).view(np.uint32) != gd[j]:
                bad += 1
                break
    return bad


def cpu_baseline(pts, queries, steps: int, check=None, lidar_gpu=None, range_gpu=None):
    """The CPU implementation (oracle_kind()) on this host's cores.

    Times batches of the headline workload on all cores and on one thread,
    the LiDAR mapping stream (kNN on all cores, mutations on one caller: the
    reference's background rebuild thread runs, calls return as the
    reference's own do), and box / radius searches on the 1M-point map on all
    cores.  `check` = (queries, xyz, d2, cnt) of GPU rows: compared row by row
    with the CPU implementation's rows on the same queries."""
    sys.path.insert(0, ORACLE)
    import oracle_lib
    kind = oracle_kind()
    cores = os.cpu_count() or 1
    t = oracle_lib.OracleTree(0.5, 0.6, DS, kind=kind)
    t.Build(pts)
    t.knn(queries[0][:1000], K, nthreads=cores)
    times = []
    for s in range(steps):
        t0 = time.perf_counter()
        t.knn(queries[s % len(queries)], K, nthreads=cores)
        times.append(time.perf_counter() - t0)
    qps = N_Q / statistics.median(times)
    # one thread, on a 20k-query slice of the same batches
    t1 = []
    for s in range(steps):
        t0 = time.perf_counter()
        t.knn(queries[s % len(queries)][:20000], K, nthreads=1)
        t1.append(time.perf_counter() - t0)
    qps_1 = 20000 / statistics.median(t1)
    out = {"value": qps, "unit": "queries/s", "cores": cores, "kind": KIND_NAME[kind], "value_1_thread": qps_1,
           "sample": f"{steps} batches of {N_Q} kNN queries (k={K}) on the 1M map, OpenMP over queries "
                     f"(1 thread: 20k-query slices); {LIDAR_SCANS} LiDAR scans on the {LIDAR_MAP}-point map; "
                     f"{RANGE_Q} box and {RANGE_Q} radius queries on the 1M map"}
    if check is not None:
        cq, gx, gd, gc = check
        rx, rd, rc = t.knn(cq, K, nthreads=cores)
        bad = knn_rows_match(cq, rx, rd, rc, gx, gd, gc)
        out["parity_sample"] = {"rows": len(cq), "rows_differing": bad, "against": KIND_NAME[kind]}
    # box / radius search on all cores
    boxes, centres, radius = range_queries()
    t0 = time.perf_counter()
    offs_b, _ = t.box_search(boxes, nthreads=cores)
    box_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    offs_r, _ = t.radius_search(centres, radius, nthreads=cores)
    rad_s = time.perf_counter() - t0
    out["range"] = {"box_queries_per_s": RANGE_Q / box_s, "radius_queries_per_s": RANGE_Q / rad_s,
                    "box_hits": int(offs_b[-1]), "radius_hits": int(offs_r[-1])}
    if range_gpu is not None:
        # box hits are shape-independent in both; the reference's radius search
        # takes whole subtrees by a sqrt bound that can admit or drop points
        # within an ulp of the radius depending on its tree shape
        out["range"]["box_hits_match_gpu"] = int(offs_b[-1]) == range_gpu["box_hits"]
        out["range"]["radius_hits_minus_gpu"] = int(offs_r[-1]) - range_gpu["radius_hits"]
    t.close()
    # LiDAR mapping stream: kNN over all cores, mutations on one caller (the
    # reference's mutations are single-caller); caller-visible times.
    base, scans = lidar_workload()
    t = oracle_lib.OracleTree(0.5, 0.6, DS, kind=kind)
    t.Build(base)
    t.set_async(True)
    upd = run_scans(t, scans, lambda p: t.knn(p, K, 5.0, nthreads=cores))
    t.set_async(False)
    upd["final_validnum"] = t.validnum()
    if lidar_gpu is not None:
        upd["final_validnum_matches_gpu"] = upd["final_validnum"] == lidar_gpu
    t.close()
    out.update(upd)
    return out


def run_reference(args):
    """The reference arm: the CPU implementation alone, on all host cores,
    one step = one 100k-query batch of the headline workload."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, ORACLE)
    import oracle_lib
    kind = oracle_kind()
    cores = os.cpu_count() or 1
    pts = make_map()
    with StdoutToStderr():
        t = oracle_lib.OracleTree(0.5, 0.6, DS, kind=kind)
        t.Build(pts)
        for s in range(args.warmup):
            t.knn(make_queries(s), K, nthreads=cores)
        times = []
        for s in range(args.steps):
            q = make_queries(args.warmup + s)
            t0 = time.perf_counter()
            t.knn(q, K, nthreads=cores)
            times.append(time.perf_counter() - t0)
        t.close()
    ms = 1e3 * statistics.mean(times)
    value = N_Q / (ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(CONFIG),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "queries/s", "cores": cores, "kind": KIND_NAME[kind],
                         "sample": f"{args.steps} timed batches of {N_Q} kNN queries (k={K}) on the 1M map, "
                                   f"OpenMP over Nearest_Search calls on {cores} threads"},
        "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def aggregate_replicas(ms: float, e2e_ms: float, units: int, world: int):
    """Replicas: every rank processed `units` per step; the job's step time
    is the slowest rank's (all-reduce MAX over the default process group when
    world > 1) and the value is the units of all ranks over that time."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms, e2e_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, e2e_ms = float(t[0]), float(t[1])
    return ms, e2e_ms, world * units / (ms / 1e3), world * units / (e2e_ms / 1e3)


def run_ours(args):
    import torch
    import torch.distributed as dist
    import ikdg

    world, rank, local = dist_env()
    if world > 1 and not dist.is_initialized():
        dist.init_process_group("gloo")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    def barrier():
        if world > 1:
            dist.barrier()

    tree = ikdg.KDTree(0.5, 0.6, DS, device=local)
    pts = make_map()
    tree.Build(pts)
    stream = torch.cuda.ExternalStream(tree.stream(), device=dev)
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device=dev)  # 512 MB > L2
    W, Kst = args.warmup, args.steps
    qhost = [make_queries(s) for s in range(W + Kst)]
    qdev = [torch.from_numpy(q).to(dev) for q in qhost]
    ids = torch.empty((N_Q, K), dtype=torch.int32, device=dev)
    d2 = torch.empty((N_Q, K), dtype=torch.float32, device=dev)
    xyz = torch.empty((N_Q, K, 3), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    def dev_step(s):
        tree.knn_device(qdev[s].data_ptr(), N_Q, K, math.inf, ids.data_ptr(), d2.data_ptr(), xyz.data_ptr())

    for s in range(W):
        dev_step(s)
    tree.synchronize()

    # ---- value: device-resident queries, per-step CUDA events on the tree stream
    barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    evs = []
    t_wall0 = time.perf_counter()
    for s in range(Kst):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            dev_step(W + s)
            e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    clocks = sampler.stop()
    barrier()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    ms = statistics.mean(step_ms)
    # rows of the last timed step, checked against the CPU implementation in
    # the cpu_baseline leg
    last_q = qhost[W + Kst - 1][:PARITY_SAMPLE]
    last_ids = ids[:PARITY_SAMPLE].cpu().numpy()
    parity_rows = (last_q, xyz[:PARITY_SAMPLE].cpu().numpy(), d2[:PARITY_SAMPLE].cpu().numpy(),
                   (last_ids >= 0).sum(1))

    # ---- e2e: pinned host buffers through the C ABI (ikdg_knn): the queries
    # come from host memory and ids, squared distances, points and counts go
    # back to host memory inside the timed call.
    qpin = [torch.from_numpy(q).pin_memory() for q in qhost]
    h_ids = torch.empty((N_Q, K), dtype=torch.int32).pin_memory()
    h_d2 = torch.empty((N_Q, K), dtype=torch.float32).pin_memory()
    h_xyz = torch.empty((N_Q, K, 3), dtype=torch.float32).pin_memory()
    h_cnt = torch.empty((N_Q,), dtype=torch.int32).pin_memory()

    def host_step(s):
        tree.knn_into(qpin[s].data_ptr(), N_Q, K, math.inf, h_ids.data_ptr(), h_d2.data_ptr(), h_xyz.data_ptr(),
                      h_cnt.data_ptr())

    for s in range(W):
        host_step(s)
    e2e_ms = []
    for s in range(Kst):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_step(W + s)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_step = statistics.mean(e2e_ms)

    # ---- LiDAR mapping stream (host API, synchronous)
    base, scans = lidar_workload()
    lt = ikdg.KDTree(0.5, 0.6, DS, device=local)
    lt.Build(base)
    lidar = run_scans(lt, scans, lambda p: lt.knn(p, K, 5.0, want_xyz=True))
    lidar["final_validnum"] = lt.validnum()
    lt.close()

    # ---- box / radius search on the headline map (device buffers)
    rng_gpu = range_bench(tree, torch, dev)
    # ---- per-point calls through the C++ facade (own process, same GPU)
    facade = facade_bench() if world == 1 else None

    # ---- batched multi-map workload, scale stress
    batched = None if args.no_batch else multimap_bench(ikdg, torch, local)
    stress = None if args.no_stress else stress_bench(ikdg, torch, local)

    # ---- aggregate over ranks (max time, summed throughput)
    ms, e2e_step, value, e2e_value = aggregate_replicas(ms, e2e_step, N_Q, world)
    peak, peak_kind = measured_peak()
    achieved = N_Q * bytes_per_query(N_MAP, K) / (ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": Kst, "warmup": W,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": dict(CONFIG),
        "parallelism": f"replicas x{world}",
        "e2e": {"value": e2e_value, "unit": "queries/s", "ms_per_step": e2e_step,
                "h2d_bytes_per_step": N_Q * 12, "d2h_bytes_per_step": N_Q * K * (4 + 4 + 12) + N_Q * 4,
                "host_buffers": "pinned"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": knn_traffic(), "peak_source": peak_kind,
                     "bytes_per_query": bytes_per_query(N_MAP, K)},
        "clocks": clocks,
        # one knn_kernel launch per timed step (query binning is off by
        # default); the L2 flush between steps is a torch fill, not ours
        "gpu_launches": Kst,
        "update_ms_per_scan": lidar["update_ms_per_scan"],
        "update": {"workload": f"lidar map {LIDAR_MAP} pts, {LIDAR_SCANS} scans of ~{lidar['scan_points']} pts, "
                               "0.5 m downsampling, 200 m sliding cube", **lidar},
        "wall_s_timed_region": t_wall,
        "range": rng_gpu,
        "facade_per_point": facade,
    }
    if batched is not None:
        line["batched"] = batched
    if stress is not None:
        line["stress"] = stress
    if rank == 0 and world == 1 and not args.no_cpu:
        with StdoutToStderr():
            cb = cpu_baseline(pts, qhost[:3], 3, check=parity_rows, lidar_gpu=lidar["final_validnum"],
                              range_gpu=rng_gpu)
        line["cpu_baseline"] = cb
        ps = cb.get("parity_sample")
        line["parity_sample_ok"] = ps is not None and ps["rows_differing"] == 0
        line["update"]["cpu_ms_per_scan"] = cb["update_ms_per_scan"]
        line["update"]["final_validnum_matches_cpu"] = cb.get("final_validnum_matches_gpu")
        rng_gpu["cpu_box_queries_per_s"] = cb["range"]["box_queries_per_s"]
        rng_gpu["cpu_radius_queries_per_s"] = cb["range"]["radius_queries_per_s"]
        rng_gpu["box_ratio_vs_cpu"] = rng_gpu["box_queries_per_s"] / cb["range"]["box_queries_per_s"]
        rng_gpu["radius_ratio_vs_cpu"] = rng_gpu["radius_queries_per_s"] / cb["range"]["radius_queries_per_s"]
        rng_gpu["box_hits_match_cpu"] = cb["range"].get("box_hits_match_gpu")
        rng_gpu["cpu_radius_hits_minus_gpu"] = cb["range"].get("radius_hits_minus_gpu")
        if facade and "us_per_call_1_thread" in facade:
            facade["cpu_us_per_call_1_thread"] = 1e6 / cb["value_1_thread"]
            facade["cpu_calls_per_s_all_cores"] = cb["value"]
            facade["cpu_cores"] = cb["cores"]
    if rank == 0:
        print(json.dumps(line), flush=True)
    tree.close()
    if world > 1:
        dist.destroy_process_group()


def run_leg(args):
    """One leg alone (for profiling): prints its JSON object."""
    import torch
    import ikdg
    torch.cuda.set_device(0)
    if args.leg == "knn":
        # the headline step alone: `warmup` device steps (queries and results
        # in HBM), then `steps` end-to-end steps (pinned host buffers, results
        # written by the kernel)
        tree = ikdg.KDTree(0.5, 0.6, DS)
        tree.Build(make_map())
        dev = torch.device("cuda", 0)
        qh = make_queries(0)
        q = torch.from_numpy(qh).to(dev)
        ids = torch.empty((N_Q, K), dtype=torch.int32, device=dev)
        d2 = torch.empty((N_Q, K), dtype=torch.float32, device=dev)
        xyz = torch.empty((N_Q, K, 3), dtype=torch.float32, device=dev)
        for _ in range(args.warmup):
            tree.knn_device(q.data_ptr(), N_Q, K, math.inf, ids.data_ptr(), d2.data_ptr(), xyz.data_ptr())
        tree.synchronize()
        qp = torch.from_numpy(qh).pin_memory()
        h = [torch.empty(sh, dtype=dt).pin_memory() for sh, dt in (((N_Q, K), torch.int32), ((N_Q, K), torch.float32),
                                                                    ((N_Q, K, 3), torch.float32), ((N_Q,), torch.int32))]
        ts = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            tree.knn_into(qp.data_ptr(), N_Q, K, math.inf, *(x.data_ptr() for x in h))
            ts.append(1e3 * (time.perf_counter() - t0))
        same = bool((h[0].numpy() == ids.cpu().numpy()).all() and (h[1].numpy() == d2.cpu().numpy()).all())
        out = {"e2e_ms": statistics.median(ts), "host_rows_equal_device_rows": same}
        del qp, h
        tree.close()
    elif args.leg == "lidar":
        base, scans = lidar_workload()
        t = ikdg.KDTree(0.5, 0.6, DS)
        t.Build(base)
        out = run_scans(t, scans, lambda p: t.knn(p, K, 5.0, want_xyz=True))
        t.close()
    elif args.leg == "batch":
        out = multimap_bench(ikdg, torch, 0, reps=2, tune=False)
    else:
        out = stress_bench(ikdg, torch, 0, reps=1)
    print(json.dumps({"leg": args.leg, **out}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the multi-map batch leg")
    ap.add_argument("--no-stress", action="store_true", help="skip the 20M-point scale leg")
    ap.add_argument("--leg", choices=["knn", "lidar", "batch", "stress"], default=None,
                    help="run one leg alone on GPU 0 (for profiling) and print its object")
    args = ap.parse_args()
    if args.leg is not None:
        run_leg(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
