"""The whole registration path (tdm_register_pair) against the composition of
oracle stages on the same inputs: identical keypoints, FP32 descriptors within
1e-4 relative L2, identical mutual-NN pairs and identical RANSAC inlier set."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pair(scene):
    return scene.fragment_pair(20260004, n_points=150_000)


@pytest.fixture(scope="module")
def weights(oracle):
    return oracle.he_normal_weights(20260005)


def rel_l2(a, b):
    return float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b))


def test_describe_fragment_matches_stages(tdm, oracle, cuda, pair, weights):
    import torch
    pts = pair[0]
    net = tdm.Net(weights, precision="fp32")
    pipe = tdm.Pipeline(net, max_keypoints=64)
    kp, desc, g = pipe.describe(torch.from_numpy(pts).to(cuda), seed=41, k=64)
    dim, origin = oracle.grid_setup(pts)
    assert tuple(g.dim) == tuple(dim.tolist())
    idx = oracle.keypoint_indices(41, pts.shape[0], 64)
    ref_kp, ref_kg = oracle.keypoints(pts, idx, origin, 0.01)
    assert np.array_equal(kp.cpu().numpy(), ref_kp)
    # the TDF stage itself is checked against the brute-force oracle elsewhere
    tdf = tdm.tdf(torch.from_numpy(pts).to(cuda), g).cpu().numpy()
    patches = oracle.gather(tdf, dim, ref_kg)
    want = oracle.net_forward(patches, weights)
    assert rel_l2(desc.cpu().numpy(), want) <= 1e-4


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_register_pair_matches_stage_composition(tdm, oracle, cuda, pair, weights, prec):
    import torch
    a, b, Rt_gt = pair
    k = 1000
    net = tdm.Net(weights, precision=prec)
    pipe = tdm.Pipeline(net, max_keypoints=k, ransac_seed=20260000, ransac_iters=100000,
                        match_precision="fp32")
    da, db = torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda)
    res = pipe.register(da, db, seed=100, k=k)
    # same path from the stage calls
    descs, kps = [], []
    for f, (pts, seed) in enumerate(((a, 100), (b, 101))):
        pd = torch.from_numpy(pts).to(cuda)
        g = tdm.grid_from_points_host(pts)
        t = tdm.tdf(pd, g)
        idx = tdm.keypoint_indices(seed, pts.shape[0], k, device=cuda)
        kp, kg = tdm.keypoints(pd, idx, g)
        descs.append(net.forward(tdm.gather(t, g, kg)))
        kps.append(kp)
    d_all = torch.cat(descs).cpu().numpy()
    ref_pairs, _, _ = oracle.mutual_nn(d_all[:k], d_all[k:])
    assert res.n_matches == len(ref_pairs)
    x = kps[0].cpu().numpy()[ref_pairs[:, 0]]
    y = kps[1].cpu().numpy()[ref_pairs[:, 1]]
    ref = oracle.ransac(x, y, seed=20260000, iters=100000, thr=0.05)
    assert res.best_trial == ref["best_trial"]
    assert res.n_inliers == len(ref["inliers"])
    rt = np.array(res.rt).reshape(4, 4)
    assert np.abs(rt[:3] - ref["Rt"]).max() < 1e-9
    tdm.device_status()


def test_register_pair_host_equals_device(tdm, cuda, pair, weights):
    import torch
    a, b, _ = pair
    net = tdm.Net(weights, precision="bf16")
    pipe = tdm.Pipeline(net, max_keypoints=500, ransac_iters=20000, match_precision="bf16")
    r_dev = pipe.register(torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda), seed=7, k=500)
    r_host = pipe.register(a, b, seed=7, k=500)
    assert r_dev.n_matches == r_host.n_matches and r_dev.best_trial == r_host.best_trial
    assert np.array_equal(np.array(r_dev.rt), np.array(r_host.rt))


def test_bf16_nearest_neighbours_agree_where_fp32_separates_them(tdm, oracle, cuda, pair, weights):
    """Real pipeline descriptors of C1 shape (1,000 keypoints on each fragment
    of a synthetic pair, 30^3 patches, random He-normal weights): wherever the
    FP32 form's nearest neighbour is more than 5 % closer than its second
    (second / first distance > 1.05, exact FP64 distances), the BF16 form --
    BF16 descriptors and the BF16 distance GEMM -- returns the same nearest
    neighbour (core/demo.m:51-57 nn), in both directions.  Random weights
    leave most descriptors nearly equidistant; the rows below the margin are
    reported, not asserted."""
    import torch
    a, b, _ = pair
    k = 1000
    nets = {p: tdm.Net(weights, precision=p) for p in ("fp32", "bf16")}
    desc = {}
    for p, net in nets.items():
        pipe = tdm.Pipeline(net, max_keypoints=k)
        da = pipe.describe(torch.from_numpy(a).to(cuda), seed=3, k=k)[1]
        db = pipe.describe(torch.from_numpy(b).to(cuda), seed=4, k=k)[1]
        desc[p] = (da, db)
        pipe.close()
    _, _, ab32, ba32 = tdm.match_mnn(*desc["fp32"], precision="fp32")
    _, _, ab16, ba16 = tdm.match_mnn(*desc["bf16"], precision="bf16")
    f32a, f32b = (x.cpu().numpy() for x in desc["fp32"])
    _, ref_ab, ref_ba = oracle.mutual_nn(f32a, f32b)
    d32a, d32b = f32a.astype(np.float64), f32b.astype(np.float64)
    report = []
    for q, r, nn32, nn16, ref in ((d32a, d32b, ab32, ab16, ref_ab), (d32b, d32a, ba32, ba16, ref_ba)):
        d2 = (q * q).sum(1)[:, None] + (r * r).sum(1)[None, :] - 2.0 * q @ r.T
        d = np.sqrt(np.maximum(d2, 0.0))
        two = np.sort(d, axis=1)[:, :2]
        margin = two[:, 1] / np.maximum(two[:, 0], 1e-30)
        sep = margin > 1.05
        nn32, nn16 = nn32.cpu().numpy(), nn16.cpu().numpy()
        assert np.array_equal(nn32, ref)  # the FP32 form is the exact NN
        assert sep.sum() >= 20
        assert np.array_equal(nn16[sep], nn32[sep]), int((nn16[sep] != nn32[sep]).sum())
        report.append((int(sep.sum()), float(np.mean(nn16 == nn32))))
    print("rows with FP32 margin > 5 %% / BF16 agreement over all rows: %s" % report)
    tdm.device_status()
