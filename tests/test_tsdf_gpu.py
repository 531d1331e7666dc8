"""GPU parity of TSDF fusion and surface extraction against the oracle
(tolerance 1e-6 absolute on TSDF values; the kernels match bit for bit)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

K = np.array([585.0, 0, 320.0, 0, 585.0, 240.0, 0, 0, 1], np.float32)


@pytest.fixture(scope="module")
def seq(scene):
    return scene.depth_sequence(20260003, n_frames=50)


def _gpu_fuse(tdm, cuda, depth_mm, poses, dim, origin, vs, trunc):
    import torch
    mm = torch.from_numpy(depth_mm.astype(np.uint16).view(np.int16)).to(cuda)
    depth = torch.empty(depth_mm.shape, dtype=torch.float32, device=cuda)
    tdm.depth_from_mm(mm, depth)
    V = int(np.prod(dim))
    ts = torch.empty(V, dtype=torch.float32, device=cuda)
    wt = torch.empty(V, dtype=torch.float32, device=cuda)
    tdm.tsdf_init(ts, wt, dim)
    tdm.tsdf_integrate(ts, wt, dim, origin, vs, trunc, depth, K, poses)
    return ts, wt, depth


def test_depth_from_mm(tdm, cuda, seq):
    import torch
    frames, _ = seq
    mm = frames[:2].copy()
    mm[0, 0, :5] = [0, 1, 5999, 6000, 6001]
    t = torch.from_numpy(mm.view(np.int16)).to(cuda)
    out = torch.empty(mm.shape, dtype=torch.float32, device=cuda)
    tdm.depth_from_mm(t, out)
    want = mm.astype(np.float32) / np.float32(1000.0)
    want[want > 6.0] = 0
    assert np.array_equal(out.cpu().numpy(), want)


def test_tsdf_small_grid_bit_exact(tdm, oracle, cuda, seq):
    frames, poses = seq
    dim = np.array([96, 80, 64], np.int32)
    origin = np.array([-1.0, -0.8, 0.6], np.float32)
    vs, trunc = 0.02, 0.1
    ts, wt, depth = _gpu_fuse(tdm, cuda, frames[:8], poses[:8], dim, origin, vs, trunc)
    rts = np.ones(int(np.prod(dim)), np.float32)
    rwt = np.zeros_like(rts)
    d = depth.cpu().numpy()
    for f in range(8):
        oracle.tsdf_integrate(K, poses[f], d[f], dim, origin, vs, trunc, rts, rwt)
    assert np.array_equal(wt.cpu().numpy(), rwt)
    assert np.abs(ts.cpu().numpy() - rts).max() <= 1e-6
    assert np.array_equal(ts.cpu().numpy(), rts)
    assert rwt.max() == 8


def test_tsdf_512_grid_50_frames(tdm, oracle, cuda, seq):
    """The 512^3 x 50-frame fusion at 6 mm; the oracle checks three z slabs."""
    frames, poses = seq
    dim = np.array([512, 512, 512], np.int32)
    origin = np.array([-1.536, -1.536, 0.5], np.float32)
    vs = 0.006
    trunc = float(np.float32(vs) * np.float32(5))
    ts, wt, depth = _gpu_fuse(tdm, cuda, frames, poses, dim, origin, vs, trunc)
    g_ts = ts.cpu().numpy().reshape(512, 512, 512)
    g_wt = wt.cpu().numpy().reshape(512, 512, 512)
    assert g_wt.max() <= 50 and g_wt.max() >= 40
    assert g_ts.min() >= -1.0 and g_ts.max() <= 1.0
    d = depth.cpu().numpy()
    for z0 in (40, 200, 380):
        rts = np.ones(int(np.prod(dim)), np.float32)
        rwt = np.zeros_like(rts)
        for f in range(50):
            oracle.tsdf_integrate(K, poses[f], d[f], dim, origin, vs, trunc, rts, rwt, z0=z0, z1=z0 + 4)
        r_ts = rts.reshape(512, 512, 512)[z0:z0 + 4]
        r_wt = rwt.reshape(512, 512, 512)[z0:z0 + 4]
        assert np.array_equal(g_wt[z0:z0 + 4], r_wt), z0
        assert np.abs(g_ts[z0:z0 + 4] - r_ts).max() <= 1e-6, z0


def test_surface_extraction(tdm, oracle, cuda, seq):
    frames, poses = seq
    dim = np.array([120, 100, 90], np.int32)
    origin = np.array([-1.2, -1.0, 0.5], np.float32)
    vs, trunc = 0.02, 0.1
    ts, wt, _ = _gpu_fuse(tdm, cuda, frames[:10], poses[:10], dim, origin, vs, trunc)
    pts, n = tdm.tsdf_extract(ts, wt, dim, origin, vs, 0.2, 1.0)
    n = int(n.item())
    want = oracle.extract_surface(ts.cpu().numpy(), wt.cpu().numpy(), dim, origin, vs, 0.2, 1.0)
    assert n == want.shape[0] and n > 1000
    assert np.array_equal(pts[:n].cpu().numpy(), want)
    # truncated output keeps the count and the first max_pts points
    pts2, n2 = tdm.tsdf_extract(ts, wt, dim, origin, vs, 0.2, 1.0, max_pts=100)
    assert int(n2.item()) == n and np.array_equal(pts2[:100].cpu().numpy(), want[:100])
