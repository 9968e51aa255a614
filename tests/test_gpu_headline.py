"""Parity at the sizes the numbers are quoted on.

* The headline workload: a 1M-point map uniform in [-50, 50]^3 (the bench's
  map seed) and one full batch of 100k uniform queries (the bench's first
  query batch), k = 5, max_dist = inf.  Every row is compared with the
  unmodified reference (where its library is built) and with the oracle port,
  whose kNN runs on all host cores.
* The plain small configuration exactly as written: a 100k-point uniform map,
  10k kNN queries (k = 5, max_dist = inf), Add_Points of 1k new uniform points
  without downsampling, Delete_Point_Boxes on 10 random boxes of side 2-10 m,
  then the same queries again.  Return values, every kNN row, validnum and
  the final set of valid points are compared with the same CPU
  implementations; ids are also compared bit for bit with the numpy model on
  the first 1,000 queries.
"""
import math
import os

import numpy as np
import pytest

import golden_check as G
import oracle_lib
import spec

pytestmark = pytest.mark.gpu

CORES = os.cpu_count() or 1


def test_headline_batch_full_size(ikdg_mod, cpu_kinds):
    pts = np.random.default_rng(1002).uniform(-50, 50, (1_000_000, 3)).astype(np.float32)
    q = np.random.default_rng(7000).uniform(-50, 50, (100_000, 3)).astype(np.float32)
    gpu = ikdg_mod.KDTree(0.5, 0.6, 0.5)
    gpu.Build(pts)
    ids, d2, xyz, cnt = gpu.knn(q, 5, math.inf)
    assert np.all(cnt == 5)
    for kind in cpu_kinds:
        cpu = oracle_lib.OracleTree(0.5, 0.6, 0.5, kind=kind)
        cpu.Build(pts)
        rxyz, rd2, rcnt = cpu.knn(q, 5, math.inf, nthreads=CORES)
        ties = G.check_knn_rows_bulk(q, rxyz, rd2, rcnt, xyz, d2, cnt)
        print(f"headline batch: 100000 rows equal to the {kind} ({ties} rows with tied distances)")
        cpu.close()
    gpu.close()


def config1_inputs():
    rng = np.random.default_rng(1001)
    pts = rng.uniform(-50, 50, (100_000, 3)).astype(np.float32)
    q = rng.uniform(-50, 50, (10_000, 3)).astype(np.float32)
    add = rng.uniform(-50, 50, (1_000, 3)).astype(np.float32)
    c = rng.uniform(-50, 50, (10, 3))
    side = rng.uniform(2, 10, (10, 3))
    boxes = np.concatenate([c - side / 2, c + side / 2], 1).astype(np.float32)
    return pts, q, add, boxes


def test_plain_small_configuration(ikdg_mod, cpu_kinds):
    pts, q, add, boxes = config1_inputs()
    gpu = ikdg_mod.KDTree(0.5, 0.6, 0.2)
    model = spec.SpecTree(0.2)
    cpus = {kind: oracle_lib.OracleTree(0.5, 0.6, 0.2, kind=kind) for kind in cpu_kinds}
    for t in (gpu, model, *cpus.values()):
        t.Build(pts)

    def compare_queries(stage):
        ids, d2, xyz, cnt = gpu.knn(q, 5, math.inf)
        mid, md2 = model.knn(q[:1000], 5, math.inf)
        assert np.array_equal(ids[:1000], mid), f"{stage}: ids differ from the model"
        assert np.array_equal(d2[:1000].view(np.uint32), md2.view(np.uint32))
        for kind, cpu in cpus.items():
            rxyz, rd2, rcnt = cpu.knn(q, 5, math.inf, nthreads=CORES)
            G.check_knn_rows_bulk(q, rxyz, rd2, rcnt, xyz, d2, cnt)

    compare_queries("after Build")
    ret = gpu.Add_Points(add, False)
    assert ret == model.Add_Points(add, False)
    for kind, cpu in cpus.items():
        assert ret == cpu.Add_Points(add, False), f"Add_Points return differs from the {kind}"
    n_del = gpu.Delete_Point_Boxes(boxes)
    assert n_del == model.Delete_Point_Boxes(boxes) and n_del > 0
    for kind, cpu in cpus.items():
        assert n_del == cpu.Delete_Point_Boxes(boxes), f"Delete_Point_Boxes count differs from the {kind}"
    compare_queries("after the updates")
    valid = gpu.flatten()
    assert gpu.validnum() == model.validnum() == len(valid)
    for kind, cpu in cpus.items():
        assert gpu.validnum() == cpu.validnum()
        assert G.same_point_set(valid, cpu.flatten()), f"valid points differ from the {kind}"
        cpu.close()
    assert gpu.validate() == 0
    gpu.close()
