"""The allocation-free kNN entry point (ikdg_knn_device_noalloc).

Some callers may not allocate device memory while they search: real-time loops
that cannot take an allocation's synchronisation and latency, and hosts whose
framework reserves all device memory itself.  They use this variant, whose
query-sort scratch is a static device array inside libikdg.  Checked through
the C ABI against the ordinary device kNN (ikdg_knn_device), bit for bit, on
two calls in a row (the second call reuses the scratch left by the first), for
register-resident (k <= 8) and shared-memory (8 < k <= 64) candidate lists.
This file is collected last so that a stop-at-first-failure run has already
run every other test.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NQ = 20000  # large enough that the batch is sorted, i.e. the scratch is used


def _device_knn(tree, fn, q, k, max_dist):
    import torch
    dev = q.device
    out = (torch.empty((len(q), k), dtype=torch.int32, device=dev),
           torch.empty((len(q), k), dtype=torch.float32, device=dev),
           torch.empty((len(q), k, 3), dtype=torch.float32, device=dev),
           torch.empty((len(q),), dtype=torch.int32, device=dev))
    fn(q.data_ptr(), len(q), k, max_dist, *(o.data_ptr() for o in out))
    tree.synchronize()
    return [o.cpu().numpy() for o in out]


def test_noalloc_knn_matches_device_knn_twice(ikdg_mod):
    import torch
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(77)
    pts = rng.uniform(-40, 40, (300000, 3)).astype(np.float32)
    tree = ikdg_mod.KDTree(device=0)
    tree.Build(pts)
    for call, (k, md) in enumerate(((5, math.inf), (8, 2.0), (16, math.inf), (64, 3.0))):
        q = torch.from_numpy(rng.uniform(-41, 41, (NQ, 3)).astype(np.float32)).to(dev)
        want = _device_knn(tree, tree.knn_device, q, k, md)
        got = _device_knn(tree, tree.knn_device_noalloc, q, k, md)
        for w, g in zip(want, got):
            assert np.array_equal(w, g), f"call {call}: results differ"
    tree.close()


def test_noalloc_rejects_oversized_batches(ikdg_mod):
    import torch
    tree = ikdg_mod.KDTree(device=0)
    tree.Build(np.zeros((10, 3), np.float32))
    n = 262144 + 1
    q = torch.zeros((n, 3), dtype=torch.float32, device="cuda:0")
    ids = torch.empty((n, 1), dtype=torch.int32, device="cuda:0")
    d2 = torch.empty((n, 1), dtype=torch.float32, device="cuda:0")
    with pytest.raises(ikdg_mod.IkdgError, match="262144"):
        tree.knn_device_noalloc(q.data_ptr(), n, 1, math.inf, ids.data_ptr(), d2.data_ptr())
    with pytest.raises(ikdg_mod.IkdgError, match="k must be"):
        tree.knn_device_noalloc(q.data_ptr(), 10, 65, math.inf, ids.data_ptr(), d2.data_ptr())
    tree.close()
