"""Cross-checks of the oracle's restated loops against independent numpy /
torch formulations (no GPU)."""
import os

import numpy as np
import pytest


def _sep_tdf(occ3, r):
    """Exact windowed squared-distance TDF via numpy min-filters (x, y, z)."""
    big = 10 ** 6
    g = np.where(occ3 > 0, 0, big).astype(np.int64)
    for axis in (2, 1, 0):
        out = np.full(g.shape, big, np.int64)
        n = g.shape[axis]
        for d in range(-r, r + 1):
            src = [slice(None)] * 3
            dst = [slice(None)] * 3
            if d >= 0:
                src[axis] = slice(d, n)
                dst[axis] = slice(0, n - d)
            else:
                src[axis] = slice(0, n + d)
                dst[axis] = slice(-d, n)
            out[tuple(dst)] = np.minimum(out[tuple(dst)], g[tuple(src)] + d * d)
        g = out
    v = (np.float32(1) - np.sqrt(g.astype(np.float32)) / np.float32(r)).astype(np.float32)
    v = np.where(g >= big, np.float32(0), np.maximum(v, np.float32(0)))
    return np.where(occ3 > 0, np.float32(1), v).astype(np.float32)


def test_tdf_brute_force_equals_separable(oracle):
    rng = np.random.default_rng(0)
    dim = np.array([37, 29, 23], np.int32)
    occ = (rng.random(int(np.prod(dim))) < 0.01).astype(np.uint8)
    t = oracle.tdf(occ, dim, 0.01, np.float32(0.01) * np.float32(5), mode=0)
    sep = _sep_tdf(occ.reshape(dim[2], dim[1], dim[0]), 5).reshape(-1)
    assert np.array_equal(t, sep)


def test_grid_and_occupancy_float_semantics(oracle):
    pts = np.array([[0.1, 0.2, 1.0], [0.35, -0.2, 1.4], [0.0049999, 0.0, 1.2]], np.float32)
    dim, origin = oracle.grid_setup(pts)
    mn = pts.min(0)
    assert np.array_equal(origin, (mn - np.float32(15) * np.float32(0.01) + np.float32(0.01) / np.float32(2)))
    occ = oracle.occupancy(pts, dim, origin, 0.01)
    assert occ.sum() == 3


def test_conv_matches_torch_float64(oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    w = oracle.he_normal_weights(11)
    patches = (rng.random((2, 27000)) * (rng.random((2, 27000)) < 0.2)).astype(np.float32)
    got = oracle.net_forward(patches, w, f64=True)
    x = torch.from_numpy(patches.astype(np.float64)).reshape(2, 1, 30, 30, 30)
    for i, n in enumerate(oracle.NET_LAYERS):
        wt = torch.from_numpy(w[n + ".weight"].astype(np.float64))
        bt = torch.from_numpy(w[n + ".bias"].reshape(-1).astype(np.float64))
        x = torch.nn.functional.conv3d(x, wt, bt)
        if i < 8:
            x = torch.relu(x)
        if i == 1:
            x = torch.nn.functional.max_pool3d(x, 2, 2, ceil_mode=True)
    want = x.reshape(2, 512).numpy()
    assert np.abs(got - want).max() < 1e-9 * max(1.0, np.abs(want).max())
    f32 = oracle.net_forward(patches, w)
    assert np.linalg.norm(f32 - want) / np.linalg.norm(want) < 1e-5


def test_mutual_nn_bruteforce(oracle):
    rng = np.random.default_rng(2)
    a = rng.normal(size=(60, 16)).astype(np.float32)
    b = np.concatenate([a[:40] + 0.01 * rng.normal(size=(40, 16)), rng.normal(size=(30, 16))]).astype(np.float32)
    pairs, nn_ab, nn_ba = oracle.mutual_nn(a, b)
    d = ((a[:, None, :].astype(np.float64) - b[None, :, :].astype(np.float64)) ** 2).sum(-1)
    assert np.array_equal(nn_ab, d.argmin(1))
    assert np.array_equal(nn_ba, d.argmin(0))
    want = [(nn_ba[j], j) for j in range(len(b)) if nn_ab[nn_ba[j]] == j]
    assert pairs.tolist() == [list(p) for p in want]
    assert len(pairs) >= 40


def test_ransac_samples_distinct_and_in_range(oracle):
    for m in (3, 4, 7, 1000):
        for h in range(200):
            s = oracle.ransac_sample(99, h, m)
            assert len(set(s.tolist())) == 3 and s.min() >= 0 and s.max() < m


def test_ransac_recovers_transform(oracle):
    rng = np.random.default_rng(3)
    y = rng.uniform(-1, 1, (300, 3)).astype(np.float32)
    ang = 0.4
    R = np.array([[np.cos(ang), -np.sin(ang), 0], [np.sin(ang), np.cos(ang), 0], [0, 0, 1]])
    t = np.array([0.3, -0.2, 0.1])
    x = (y @ R.T + t).astype(np.float32)
    x[200:] = rng.uniform(-1, 1, (100, 3))  # outliers
    res = oracle.ransac(x, y, seed=5, iters=2000, thr=0.05, want_counts=True)
    assert np.abs(res["Rt"][:, :3] - R).max() < 1e-5
    assert np.abs(res["Rt"][:, 3] - t).max() < 1e-5
    assert set(range(200)) <= set(res["inliers"].tolist())
    # tie rule: the winner is the latest trial with the maximum count
    c = res["counts"]
    assert res["best_trial"] == np.flatnonzero(c == c.max()).max()
    n, best = oracle.ransac_adaptive_stop(c, 300)
    assert 10 <= n <= 2000 and c[best] == c[:n].max()


def test_fp32_trial_fit_is_kabsch(oracle):
    """RANSAC's FP32 three-point fit agrees with the FP64 Kabsch fit of the same
    triple, is a proper rotation, and recovers an exact rigid motion.  The gap
    grows with the triangle's conditioning (thin triangles: FP32 resolves the
    second singular direction to ~1e-5 of s0/s1), so it is bounded relative to
    that; the median gap is ~3e-7."""
    rng = np.random.default_rng(11)
    gaps = []
    for trial in range(300):
        y = rng.uniform(-2.0, 2.0, (3, 3)).astype(np.float32)
        a = np.cross(y[1] - y[0], y[2] - y[0])
        if np.linalg.norm(a) < 0.5:  # skip near-degenerate triangles
            continue
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        ang = rng.uniform(-np.pi, np.pi)
        K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
        Rt = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
        tt = rng.uniform(-1, 1, 3)
        x = (y.astype(np.float64) @ Rt.T + tt + rng.normal(scale=0.002, size=(3, 3))).astype(np.float32)
        R32, t32 = oracle.kabsch3f(x, y, [0, 1, 2])
        R64, t64 = oracle.kabsch(x, y)
        gap = max(float(np.abs(R32 - R64).max()), float(np.abs(t32 - t64).max()))
        sv = np.linalg.svd((y - y.mean(0)).T.astype(np.float64) @ (x - x.mean(0)), compute_uv=False)
        assert gap <= 2e-5 * sv[0] / sv[1] + 1e-5, (gap, sv)
        gaps.append(gap)
        assert abs(np.linalg.det(R32.astype(np.float64)) - 1.0) < 1e-5
        assert np.abs(R32.astype(np.float64) @ R32.T - np.eye(3)).max() < 1e-5
    assert np.median(gaps) < 2e-6, np.median(gaps)
    # exact data: the motion itself
    y = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0.5]], np.float32)
    R = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], np.float64)
    x = (y @ R.T + np.array([0.5, -0.25, 1.0])).astype(np.float32)
    R32, t32 = oracle.kabsch3f(x, y, [0, 1, 2])
    assert np.abs(R32 - R).max() < 1e-6 and np.abs(t32 - [0.5, -0.25, 1.0]).max() < 1e-6


def test_marvin_roundtrip(oracle, tmp_path):
    w = oracle.he_normal_weights(4)
    p = str(tmp_path / "w.marvin")
    oracle.write_marvin(p, w)
    r = oracle.read_marvin(p)
    for k in w:
        assert np.array_equal(r[k], w[k])
    oracle.write_marvin(p, w, dtype=np.float16)
    r = oracle.read_marvin(p)
    assert np.abs(r["conv3.weight"] - w["conv3.weight"]).max() < 1e-3


def test_ply_roundtrip(oracle, tmp_path):
    pts = np.random.default_rng(5).normal(size=(100, 3)).astype(np.float32)
    p = str(tmp_path / "c.ply")
    oracle.write_ply(p, pts)
    assert np.array_equal(oracle.read_ply(p), pts)


def test_tsdf_single_frame_plane(oracle):
    """A fronto-parallel wall at 1 m: voxels just in front of it get positive
    values, behind it are skipped beyond -trunc, on it ~0."""
    H, W = 48, 64
    K = np.array([[50.0, 0, 32], [0, 50.0, 24], [0, 0, 1]], np.float32)
    depth = np.full((H, W), 1.0, np.float32)
    dim = np.array([16, 16, 16], np.int32)
    origin = np.array([-0.08, -0.08, 0.92], np.float32)
    ts = np.ones(int(np.prod(dim)), np.float32)
    wt = np.zeros_like(ts)
    oracle.tsdf_integrate(K, np.eye(4, dtype=np.float32), depth, dim, origin, 0.01, 0.05, ts, wt)
    g = ts.reshape(16, 16, 16)
    assert wt.max() == 1
    assert abs(g[8, 8, 8]) < 0.05  # z = 1.0 m
    assert g[3, 8, 8] > 0.9        # 5 cm in front
    pts = oracle.extract_surface(ts, wt, dim, origin, 0.01, 0.2, 0.0)
    assert len(pts) > 0 and np.all(np.abs(pts[:, 2] - 1.0) < 0.011)
