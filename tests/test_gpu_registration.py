"""Differentiable scan-to-map registration on the kNN result.

A 1M-point planar map (ground + walls, as in the LiDAR workload), a 20k-point
scan seen from a pose perturbed by rotation sigma = 2 deg and translation
sigma = 0.3 m.  The GPU forward (kNN k = 5 -> least-squares plane per
neighbourhood -> point-to-plane residuals, L = 1/2 sum r^2) and the
hand-written adjoint (neighbours held fixed) are checked against

* FP64 central finite differences (h = 1e-6) of the same loss, and
* an FP64 analytic gradient (numpy; Eigen is not installed here, numpy float64
  stands in for the CPU Eigen reference),

to within 1e-4 relative error, for the 6-DoF pose and for the scan points.
The torch.autograd.Function below exists only in this test harness.
"""
import math

import numpy as np
import pytest

import synthetic as S

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

K = 5
MAX_DIST = 5.0
THRESH = 0.1


def so3_exp(w):
    w = np.asarray(w, np.float64)
    th = np.linalg.norm(w)
    Kx = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-6:
        a, b = 1 - th * th / 6, 0.5 - th * th / 24
    else:
        a, b = math.sin(th) / th, (1 - math.cos(th)) / th ** 2
    return np.eye(3) + a * Kx + b * Kx @ Kx


def so3_log(R):
    c = np.clip((np.trace(R) - 1) / 2, -1, 1)
    th = math.acos(c)
    v = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    return v * (0.5 if th < 1e-8 else th / (2 * math.sin(th)))


def so3_jr(w):
    w = np.asarray(w, np.float64)
    th = np.linalg.norm(w)
    Kx = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-4:
        a, b = 0.5 - th * th / 24, 1 / 6 - th * th / 120
    else:
        a, b = (1 - math.cos(th)) / th ** 2, (th - math.sin(th)) / th ** 3
    return np.eye(3) - a * Kx + b * Kx @ Kx


def residual64(pose, p, planes):
    """r = n . (w - c) with planes[i] = {n, d, c, 0}."""
    R = so3_exp(pose[:3])
    w = p @ R.T + pose[3:]
    return (planes[:, 0:3] * (w - planes[:, 4:7])).sum(1)


def loss64(pose, p, planes, valid):
    r = residual64(pose, p, planes)
    return 0.5 * float((r[valid] ** 2).sum())


def analytic64(pose, p, planes, valid):
    R = so3_exp(pose[:3])
    r = residual64(pose, p, planes)
    g = np.where(valid[:, None], r[:, None] * planes[:, :3], 0.0)
    v = g @ R                     # rows: R^T g_i
    grad_t = g.sum(0)
    grad_w = so3_jr(pose[:3]).T @ np.cross(p, v).sum(0)
    return np.concatenate([grad_w, grad_t]), v


class P2PLoss(torch.autograd.Function):
    """loss = 1/2 sum r^2 as a differentiable function of (pose, points)."""

    @staticmethod
    def forward(ctx, pose, points, tree):
        n = points.shape[0]
        dev = points.device
        planes = torch.empty((n, 8), dtype=torch.float32, device=dev)
        res = torch.empty((n,), dtype=torch.float32, device=dev)
        valid = torch.empty((n,), dtype=torch.int32, device=dev)
        pz = pose.detach().cpu().double().tolist()
        loss = tree.p2p_forward(points.data_ptr(), n, pz, K, MAX_DIST, THRESH, planes.data_ptr(), res.data_ptr(),
                                valid.data_ptr())
        ctx.save_for_backward(points, planes, res, valid)
        ctx.pose = pz
        ctx.tree = tree
        return torch.tensor(loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        points, planes, res, valid = ctx.saved_tensors
        gp = torch.empty_like(points)
        g = ctx.tree.p2p_adjoint(points.data_ptr(), points.shape[0], ctx.pose, planes.data_ptr(), res.data_ptr(),
                                 valid.data_ptr(), float(grad_out), gp.data_ptr())
        ctx.tree.synchronize()
        return torch.tensor(g, dtype=torch.float64), gp, None


@pytest.fixture(scope="module")
def scene(ikdg_mod):
    world = S.lidar_world(4001)
    base = S.lidar_map(world, 1_000_000, 4002)
    tree = ikdg_mod.KDTree(0.5, 0.6, 0.5)
    tree.Build(base)
    poses = S.trajectory(2, 4003)
    px, py, yaw = poses[0]
    scan_w = np.concatenate([S.lidar_scan(world, poses[0], 4100), S.lidar_scan(world, poses[1], 4101)])[:20000]
    R_true = so3_exp([0, 0, yaw])
    t_true = np.array([px, py, 1.8])
    p_body = ((scan_w - t_true) @ R_true).astype(np.float32)   # R^T (s - t)
    rng = np.random.default_rng(4004)
    R0 = R_true @ so3_exp(rng.normal(0, math.radians(2.0), 3))
    t0 = t_true + rng.normal(0, 0.3, 3)
    pose0 = np.concatenate([so3_log(R0), t0])
    return tree, p_body, pose0


def test_pose_and_point_gradients_match_fp64(scene):
    tree, p, pose = scene
    dev = torch.device("cuda", 0)
    pts = torch.from_numpy(p).to(dev)
    n = len(p)
    planes = torch.empty((n, 8), dtype=torch.float32, device=dev)
    res = torch.empty((n,), dtype=torch.float32, device=dev)
    valid = torch.empty((n,), dtype=torch.int32, device=dev)
    loss = tree.p2p_forward(pts.data_ptr(), n, pose, K, MAX_DIST, THRESH, planes.data_ptr(), res.data_ptr(),
                            valid.data_ptr())
    gp = torch.empty_like(pts)
    g = np.array(tree.p2p_adjoint(pts.data_ptr(), n, pose, planes.data_ptr(), res.data_ptr(), valid.data_ptr(), 1.0,
                                  gp.data_ptr()))
    tree.synchronize()
    P = planes.cpu().numpy().astype(np.float64)
    V = valid.cpu().numpy().astype(bool)
    p64 = p.astype(np.float64)
    assert V.sum() > 0.5 * n, "too few planar neighbourhoods"
    assert abs(loss - loss64(pose, p64, P, V)) <= 1e-4 * loss
    # the stored {n, d} and c describe the same plane
    assert np.abs((P[V, 0:3] * P[V, 4:7]).sum(1) + P[V, 3]).max() < 1e-3

    # FP64 central differences, h = 1e-6
    h = 1e-6
    fd = np.zeros(6)
    for j in range(6):
        e = np.zeros(6)
        e[j] = h
        fd[j] = (loss64(pose + e, p64, P, V) - loss64(pose - e, p64, P, V)) / (2 * h)
    ana, v64 = analytic64(pose, p64, P, V)
    scale = np.linalg.norm(fd)
    assert np.linalg.norm(g - fd) <= 1e-4 * scale, (g, fd)
    assert np.abs(g - fd).max() <= 1e-4 * scale
    assert np.linalg.norm(g - ana) <= 1e-4 * np.linalg.norm(ana)

    # point gradients: analytic FP64 everywhere, finite differences on a sample
    gpn = gp.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(gpn - v64) <= 1e-4 * np.linalg.norm(v64)
    rng = np.random.default_rng(5)
    for i in rng.choice(np.flatnonzero(V), 12, replace=False):
        for a in range(3):
            q = p64.copy()
            q[i, a] += h
            lp = loss64(pose, q, P, V)
            q[i, a] -= 2 * h
            lm = loss64(pose, q, P, V)
            d = (lp - lm) / (2 * h)
            assert abs(gpn[i, a] - d) <= 1e-4 * max(abs(d), np.abs(v64[i]).max(), 1e-6)


def test_autograd_function_descends(scene):
    tree, p, pose = scene
    dev = torch.device("cuda", 0)
    pts = torch.from_numpy(p).to(dev).requires_grad_(True)
    x = torch.tensor(pose, dtype=torch.float64, requires_grad=True)
    l0 = P2PLoss.apply(x, pts, tree)
    l0.backward()
    assert x.grad is not None and pts.grad is not None and torch.isfinite(pts.grad).all()
    # gradient steps on the pose with a backtracking line search (the
    # neighbours are found again at every pose)
    cur = x.detach().clone()
    first = cur_loss = float(l0)
    for _ in range(3):
        xi = cur.clone().requires_grad_(True)
        P2PLoss.apply(xi, pts.detach(), tree).backward()
        d = xi.grad / max(float(xi.grad.norm()), 1e-12)
        for alpha in (1e-2, 3e-3, 1e-3, 3e-4, 1e-4):
            cand = cur - alpha * d
            lc = float(P2PLoss.apply(cand, pts.detach(), tree))
            if lc < cur_loss:
                cur, cur_loss = cand, lc
                break
    assert cur_loss < first


def rotation_like_library(pose):
    """R(omega) in the operation order of the library's host code (Rodrigues,
    [w]x^2 by explicit sums), so the transformed points round the same way."""
    w = [float(v) for v in pose[:3]]
    th = math.sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2])
    if th < 1e-6:
        a, b = 1.0 - th * th / 6.0, 0.5 - th * th / 24.0
    else:
        a, b = math.sin(th) / th, (1.0 - math.cos(th)) / (th * th)
    Kx = [0.0, -w[2], w[1], w[2], 0.0, -w[0], -w[1], w[0], 0.0]
    K2 = [0.0] * 9
    for r in range(3):
        for c in range(3):
            s = 0.0
            for m in range(3):
                s += Kx[3 * r + m] * Kx[3 * m + c]
            K2[3 * r + c] = s
    return [(1.0 if i % 4 == 0 else 0.0) + a * Kx[i] + b * K2[i] for i in range(9)]


def test_plane_fit_and_residuals_match_fp64(scene, ikdg_mod):
    """The forward pass pinned independently of the GPU's own planes: every
    scan point is transformed as the kernel does, its k = 5 neighbours come
    from the oracle port, and an FP64 least-squares fit (QR, the way
    FAST-LIO2's Eigen solve does it) gives the plane, the validity (every
    neighbour within the threshold) and the residual, which the GPU's
    planes, flags and residuals must match."""
    import oracle_lib
    tree, p, pose = scene
    dev = torch.device("cuda", 0)
    n = len(p)
    pts = torch.from_numpy(p).to(dev)
    planes = torch.empty((n, 8), dtype=torch.float32, device=dev)
    res = torch.empty((n,), dtype=torch.float32, device=dev)
    valid = torch.empty((n,), dtype=torch.int32, device=dev)
    tree.p2p_forward(pts.data_ptr(), n, pose, K, MAX_DIST, THRESH, planes.data_ptr(), res.data_ptr(),
                     valid.data_ptr())
    tree.synchronize()
    P = planes.cpu().numpy().astype(np.float64)
    V = valid.cpu().numpy().astype(bool)
    R = rotation_like_library(pose)
    p64 = p.astype(np.float64)
    w64 = np.stack([((R[3 * r] * p64[:, 0] + R[3 * r + 1] * p64[:, 1]) + R[3 * r + 2] * p64[:, 2]) + pose[3 + r]
                    for r in range(3)], 1)
    w32 = w64.astype(np.float32)
    if not oracle_lib.available("port"):
        oracle_lib.build("port")
    cpu = oracle_lib.OracleTree(0.5, 0.6, 0.5, kind="port")
    cpu.Build(tree.flatten())
    nb6, d6, cnt6 = cpu.knn(w32, K + 1, MAX_DIST, nthreads=8)
    cpu.close()
    nb, cnt = nb6[:, :K], np.minimum(cnt6, K)
    full = cnt == K
    # neighbour sets that a last-bit difference in the transformed point
    # cannot change: the k-th and (k+1)-th distances are well apart
    gap = (cnt6 < K + 1) | (d6[:, K] - d6[:, K - 1] > 1e-3 * np.maximum(d6[:, K], 1e-12))
    assert not V[~full].any(), "a point with fewer than k neighbours was marked valid"
    A = nb[full].astype(np.float64)                              # [m, k, 3]
    Q, Rm = np.linalg.qr(A)
    x = np.linalg.solve(Rm, (Q.transpose(0, 2, 1) @ -np.ones((len(A), K, 1))))[..., 0]
    norm = np.linalg.norm(x, axis=1)
    n64, d64 = x / norm[:, None], 1.0 / norm
    e = np.abs((A * n64[:, None, :]).sum(2) + d64[:, None])       # [m, k]
    valid64 = (e <= THRESH).all(1)
    border = (np.abs(e - THRESH) < 1e-5).any(1)
    Vf = V[full]
    assert np.array_equal(Vf[~border], valid64[~border]), "validity differs from the FP64 fit"
    ok = valid64 & Vf
    assert ok.sum() > 0.5 * n
    # every plane the GPU accepts fits its neighbours within the threshold
    Pf = P[full]
    e_gpu = np.abs((A * Pf[:, None, 0:3]).sum(2) + Pf[:, 3:4])
    assert (e_gpu[Vf] <= THRESH + 1e-5).all(), "an accepted plane misses a neighbour"
    # Both sides solve the least squares by an orthogonal factorisation, so
    # they agree to rounding wherever A is not close to rank deficient.
    well = ok & (np.linalg.cond(A) < 1e6) & gap[full]
    assert well.sum() > 0.2 * ok.sum(), "too few well-conditioned planes to compare"
    assert np.abs(Pf[well, 0:3] - n64[well]).max() < 1e-5, "plane normals differ"
    assert (np.abs(Pf[well, 3] - d64[well]) <= 1e-5 * np.maximum(1.0, np.abs(d64[well]))).all(), "offsets differ"
    r64 = (n64 * w64[full]).sum(1) + d64
    r_gpu = res.cpu().numpy().astype(np.float64)[full]
    assert np.abs(r_gpu[well] - r64[well]).max() < 2e-4, "residuals differ from the FP64 fit"
