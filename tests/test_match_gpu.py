"""GPU parity of mutual-NN matching and RANSAC against the oracle.

MNN FP32 form: indices bit-exact against the exact double-precision NN.
MNN BF16 form (tcgen05 distance GEMM): >= 99 % index agreement; near ties
among the candidates resolved as the exact FP64 NN.
RANSAC: identical per-trial inlier counts, winner and inlier set; the FP64
Kabsch refit equal to the oracle's bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _descs(rng, na, nb, dim=512, overlap=0.6):
    a = rng.normal(size=(na, dim)).astype(np.float32)
    k = int(min(na, nb) * overlap)
    b = rng.normal(size=(nb, dim)).astype(np.float32)
    perm = rng.permutation(na)[:k]
    b[:k] = a[perm] + 0.3 * rng.normal(size=(k, dim)).astype(np.float32)
    return a, b[rng.permutation(nb)]


def _run(tdm, cuda, a, b, prec):
    import torch
    da = torch.from_numpy(a).to(cuda)
    db = torch.from_numpy(b).to(cuda)
    pairs, npairs, nn_ab, nn_ba = tdm.match_mnn(da, db, prec)
    n = int(npairs.item())
    return pairs[:n].cpu().numpy(), nn_ab.cpu().numpy(), nn_ba.cpu().numpy()


@pytest.mark.parametrize("na,nb", [(1000, 1000), (1, 1), (1, 7), (300, 1000), (5000, 5000)])
def test_mnn_fp32_exact(tdm, oracle, cuda, na, nb):
    rng = np.random.default_rng(na * 7 + nb)
    a, b = _descs(rng, na, nb)
    pairs, nn_ab, nn_ba = _run(tdm, cuda, a, b, "fp32")
    ref_pairs, ref_ab, ref_ba = oracle.mutual_nn(a, b)
    assert np.array_equal(nn_ab, ref_ab)
    assert np.array_equal(nn_ba, ref_ba)
    assert np.array_equal(pairs, ref_pairs)
    tdm.device_status()


def test_mnn_fp32_ties_and_near_ties(tdm, oracle, cuda):
    """Exact duplicates go to the lowest index; differences below the FP32
    expansion's resolution are still resolved exactly (full FP64 scan)."""
    rng = np.random.default_rng(5)
    a = rng.normal(size=(64, 512)).astype(np.float32)
    b = np.repeat(a[:16], 6, axis=0).copy()  # each row six times
    b[1::6, 0] = np.nextafter(b[1::6, 0], np.float32(np.inf))  # one ulp apart
    b[4::6, 7] = np.nextafter(b[4::6, 7], np.float32(-np.inf))
    b = np.concatenate([b, rng.normal(size=(20, 512)).astype(np.float32)])
    pairs, nn_ab, nn_ba = _run(tdm, cuda, a, b, "fp32")
    ref_pairs, ref_ab, ref_ba = oracle.mutual_nn(a, b)
    assert np.array_equal(nn_ab, ref_ab) and np.array_equal(nn_ba, ref_ba)
    assert np.array_equal(pairs, ref_pairs)


def test_mnn_fp32_zeros_subnormals_scales(tdm, oracle, cuda):
    """Zero and subnormal components and rows spanning many magnitudes keep
    the exact FP64 scores (the float -> double widening of every component)."""
    rng = np.random.default_rng(11)
    a = rng.normal(size=(200, 512)).astype(np.float32)
    b = a[rng.permutation(200)] + 0.2 * rng.normal(size=(200, 512)).astype(np.float32)
    a[::3, ::5] = 0.0
    b[1::4, 3::7] = 0.0
    a[::7, :16] = np.float32(1e-39)  # subnormal
    b[::5, 100:110] = np.float32(-3e-40)
    a[::11] *= np.float32(1e-12)
    b[::13] *= np.float32(1e3)
    pairs, nn_ab, nn_ba = _run(tdm, cuda, a, b, "fp32")
    ref_pairs, ref_ab, ref_ba = oracle.mutual_nn(a, b)
    assert np.array_equal(nn_ab, ref_ab) and np.array_equal(nn_ba, ref_ba)
    assert np.array_equal(pairs, ref_pairs)


@pytest.mark.parametrize("n", [1000, 5000])
def test_mnn_bf16_agreement(tdm, oracle, cuda, n):
    rng = np.random.default_rng(n)
    a, b = _descs(rng, n, n)
    pairs, nn_ab, nn_ba = _run(tdm, cuda, a, b, "bf16")
    ref_pairs, ref_ab, ref_ba = oracle.mutual_nn(a, b)
    agree = (np.mean(nn_ab == ref_ab) + np.mean(nn_ba == ref_ba)) / 2
    assert agree >= 0.99, agree
    ref_set = set(map(tuple, ref_pairs.tolist()))
    got_set = set(map(tuple, pairs.tolist()))
    assert len(ref_set & got_set) >= 0.99 * len(ref_set)


def test_mnn_bf16_rescoring_near_ties(tdm, oracle, cuda):
    """BF16 form: each of 16 queries has four near copies (an exact duplicate
    and copies one FP32 ulp nearer / farther in one component), ~2e-7 apart
    in squared distance -- inside the FP32 re-scoring's error interval, so
    those queries take the FP64 pass -- and far from every other row, so all
    four are candidates; four more queries have two exact duplicates as their
    nearest rows.  The other queries are decided in FP32.  Every index equals
    the exact FP64 nearest neighbour (duplicates: the lower index)."""
    rng = np.random.default_rng(21)
    a = rng.normal(size=(64, 512)).astype(np.float32)
    groups = []
    for i in range(16):
        e = (0.02 * rng.normal(size=512)).astype(np.float32)
        e[0] = 0.5
        b0 = a[i] + e
        near, far = b0.copy(), b0.copy()
        near[0] = np.nextafter(b0[0], a[i, 0])  # one ulp towards the query
        far[0] = np.nextafter(b0[0], np.float32(np.inf) if b0[0] > a[i, 0] else np.float32(-np.inf))
        groups.append(np.stack([b0, b0, far, near])[rng.permutation(4)])
    for i in range(16, 20):  # nearest rows are exact duplicates: the lower index wins
        e = (0.02 * rng.normal(size=512)).astype(np.float32)
        e[0] = 0.5
        b0 = a[i] + e
        far = b0.copy()
        far[0] = np.nextafter(b0[0], np.float32(np.inf) if b0[0] > a[i, 0] else np.float32(-np.inf))
        far2 = far.copy()
        far2[0] = np.nextafter(far[0], np.float32(np.inf) if far[0] > a[i, 0] else np.float32(-np.inf))
        groups.append(np.stack([far2, b0, far, b0]))
    b = np.concatenate(groups + [rng.normal(size=(20, 512)).astype(np.float32)])
    ref_pairs, ref_ab, ref_ba = oracle.mutual_nn(a, b)
    d = ((a[:16, None, :].astype(np.float64) - b[None, :64, :].astype(np.float64)) ** 2).sum(-1)
    assert len({round(x, 12) for x in d[0, :4]}) == 3  # duplicate, nearer, farther: three distances
    assert all(ref_ab[i] == 4 * i + 1 for i in range(16, 20))
    pairs, nn_ab, nn_ba = _run(tdm, cuda, a, b, "bf16")
    assert np.array_equal(nn_ab, ref_ab) and np.array_equal(nn_ba, ref_ba)
    assert np.array_equal(pairs, ref_pairs)
    tdm.device_status()


def _correspondences(rng, m, inlier_frac=0.4, noise=0.01):
    y = rng.uniform(-1.5, 1.5, (m, 3)).astype(np.float32)
    ang = 0.5
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    Kx = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + np.sin(ang) * Kx + (1 - np.cos(ang)) * Kx @ Kx
    t = np.array([0.3, -0.4, 0.2])
    x = (y @ R.T + t + noise * rng.normal(size=(m, 3))).astype(np.float32)
    k = int(m * inlier_frac)
    x[k:] = rng.uniform(-1.5, 1.5, (m - k, 3)).astype(np.float32)
    return x, y, R, t


def _ransac_gpu(tdm, cuda, x, y, m, iters, seed, adaptive=False):
    import torch
    xd = torch.from_numpy(x).to(cuda)
    yd = torch.from_numpy(y).to(cuda)
    md = torch.tensor([m], dtype=torch.int32, device=cuda)
    rt, inl, info = tdm.ransac(xd, yd, md, seed, iters, 0.05, adaptive=adaptive)
    info = info.cpu().numpy()
    return rt.cpu().numpy().reshape(3, 4), inl.cpu().numpy()[:info[0]], info


@pytest.mark.parametrize("m,iters", [(500, 100000), (37, 5000), (4000, 20000)])
def test_ransac_identical_to_oracle(tdm, oracle, cuda, m, iters):
    rng = np.random.default_rng(m)
    x, y, R, t = _correspondences(rng, m)
    rt, inl, info = _ransac_gpu(tdm, cuda, x, y, m, iters, seed=20260000)
    ref = oracle.ransac(x, y, seed=20260000, iters=iters, thr=0.05)
    assert info[1] == ref["best_trial"]
    assert np.array_equal(inl, ref["inliers"])
    assert np.abs(rt - ref["Rt"]).max() < 1e-9
    assert np.abs(rt[:, :3] - R).max() < 0.02 and np.abs(rt[:, 3] - t).max() < 0.02
    tdm.device_status()


@pytest.mark.parametrize("m,frac,noise", [(60, 0.3, 0.01), (500, 0.9, 0.005), (4000, 0.95, 0.01),
                                           (300, 0.5, 0.0)])
def test_ransac_refit_bits_equal_oracle(tdm, oracle, cuda, m, frac, noise):
    """The FP64 refit (split over a warp's lanes on the device) gives the
    oracle's one-thread Kabsch bit for bit, from 18 to 3,800 inliers."""
    rng = np.random.default_rng(100 + m)
    x, y, _, _ = _correspondences(rng, m, frac, noise)
    rt, inl, info = _ransac_gpu(tdm, cuda, x, y, m, 4000, seed=77)
    ref = oracle.ransac(x, y, seed=77, iters=4000, thr=0.05)
    assert np.array_equal(inl, ref["inliers"]) and info[0] >= 3
    assert rt.tobytes() == np.ascontiguousarray(ref["Rt"], np.float64).tobytes()


def test_ransac_trial_counts_identical(tdm, oracle, cuda):
    """Every trial's inlier count matches (read from the documented workspace
    layout: counts follow an 8-byte best word padded to 256 bytes)."""
    import ctypes
    import torch
    rng = np.random.default_rng(11)
    m, iters = 700, 30000
    x, y, _, _ = _correspondences(rng, m, 0.2)
    xd, yd = torch.from_numpy(x).to(cuda), torch.from_numpy(y).to(cuda)
    md = torch.tensor([m], dtype=torch.int32, device=cuda)
    nws = tdm.lib().tdm_ransac_workspace_bytes(m, iters)
    ws = torch.zeros(nws, dtype=torch.uint8, device=cuda)
    rt = torch.zeros(12, dtype=torch.float64, device=cuda)
    inl = torch.zeros(m, dtype=torch.int32, device=cuda)
    info = torch.zeros(4, dtype=torch.int32, device=cuda)
    prm = tdm.RansacParams(3, iters, 0.05, 0, 50000)
    tdm.check(tdm.lib().tdm_ransac(xd.data_ptr(), yd.data_ptr(), md.data_ptr(), m, ctypes.byref(prm),
                                   rt.data_ptr(), inl.data_ptr(), info.data_ptr(), ws.data_ptr(), nws,
                                   torch.cuda.current_stream().cuda_stream))
    counts = ws[256:256 + 4 * iters].cpu().numpy().view(np.int32)
    ref = oracle.ransac(x, y, seed=3, iters=iters, thr=0.05, want_counts=True)
    assert np.array_equal(counts, ref["counts"])


def test_ransac_adaptive_stop(tdm, oracle, cuda):
    rng = np.random.default_rng(12)
    m = 400
    x, y, _, _ = _correspondences(rng, m, 0.6)
    rt, inl, info = _ransac_gpu(tdm, cuda, x, y, m, 50000, seed=9, adaptive=True)
    ref = oracle.ransac(x, y, seed=9, iters=50000, thr=0.05, want_counts=True)
    n, best = oracle.ransac_adaptive_stop(ref["counts"], m, 50000)
    assert info[3] == n and info[1] == best
    assert n < 1000  # 60 % inliers stop early


def test_ransac_degenerate_inputs(tdm, cuda):
    x = np.zeros((5, 3), np.float32)
    for m in (0, 2):
        rt, inl, info = _ransac_gpu(tdm, cuda, x, x, m, 100, seed=1)
        assert info[0] == 0 and np.array_equal(rt, np.hstack([np.eye(3), np.zeros((3, 1))]))


def test_pairs_to_points(tdm, cuda):
    import torch
    ka = torch.arange(30, dtype=torch.float32, device=cuda).reshape(10, 3)
    kb = -torch.arange(30, dtype=torch.float32, device=cuda).reshape(10, 3)
    pairs = torch.tensor([[3, 1], [0, 9], [7, 7]], dtype=torch.int32, device=cuda)
    n = torch.tensor([2], dtype=torch.int32, device=cuda)
    x, y = tdm.pairs_to_points(ka, kb, pairs, n)
    assert torch.equal(x[:2], ka[[3, 0]]) and torch.equal(y[:2], kb[[1, 9]])
    assert torch.count_nonzero(x[2]) == 0
