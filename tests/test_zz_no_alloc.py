"""tdm_ransac_noalloc: RANSAC for callers that cannot allocate device memory
(a foreign-function binding without a device allocator, or a serving loop that
forbids cudaMalloc after start-up).  Its scratch is a fixed array inside the
library, so it must give exactly what tdm_ransac gives with a caller
workspace, call after call, with nothing left over from the previous call.

Kept in its own file, collected last, so a run that stops at the first failure
has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_TRIALS = 131072


def _problem(seed, m, inlier_frac):
    rng = np.random.default_rng(seed)
    y = rng.uniform(-1.5, 1.5, (m, 3)).astype(np.float32)
    a = rng.uniform(0.1, 0.6)
    R = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    x = (y @ R.T + rng.normal(0, 0.01, (m, 3)) + [0.2, -0.1, 0.3]).astype(np.float32)
    k = int(m * inlier_frac)
    x[k:] = rng.uniform(-1.5, 1.5, (m - k, 3)).astype(np.float32)
    return x, y


def _call(tdm, cuda, x, y, iters, seed, noalloc):
    import torch
    lib = tdm.lib()
    m = x.shape[0]
    xd, yd = torch.from_numpy(x).to(cuda), torch.from_numpy(y).to(cuda)
    md = torch.tensor([m], dtype=torch.int32, device=cuda)
    rt = torch.full((12,), -7.0, dtype=torch.float64, device=cuda)
    inl = torch.full((m,), -1, dtype=torch.int32, device=cuda)
    info = torch.full((4,), -1, dtype=torch.int32, device=cuda)
    prm = tdm.RansacParams(seed, iters, 0.05, 0, 50000)
    s = torch.cuda.current_stream().cuda_stream
    if noalloc:
        st = lib.tdm_ransac_noalloc(xd.data_ptr(), yd.data_ptr(), md.data_ptr(), m, ctypes.byref(prm), rt.data_ptr(),
                                    inl.data_ptr(), info.data_ptr(), s)
    else:
        nws = lib.tdm_ransac_workspace_bytes(m, iters)
        ws = torch.empty(nws, dtype=torch.uint8, device=cuda)
        st = lib.tdm_ransac(xd.data_ptr(), yd.data_ptr(), md.data_ptr(), m, ctypes.byref(prm), rt.data_ptr(),
                            inl.data_ptr(), info.data_ptr(), ws.data_ptr(), nws, s)
    tdm.check(st)
    torch.cuda.synchronize()
    info = info.cpu().numpy()
    return rt.cpu().numpy(), inl.cpu().numpy()[:info[0]], info


def test_noalloc_matches_workspace_version_call_after_call(tdm, cuda):
    # three calls in a row, alternating problems: a call must not see the last one's state
    cases = [(_problem(1, 600, 0.5), 100000, 11), (_problem(2, 250, 0.2), 30000, 12), (_problem(1, 600, 0.5), 100000, 11)]
    for (x, y), iters, seed in cases:
        want = _call(tdm, cuda, x, y, iters, seed, noalloc=False)
        got = _call(tdm, cuda, x, y, iters, seed, noalloc=True)
        assert np.array_equal(got[2], want[2])
        assert np.array_equal(got[1], want[1])
        assert np.abs(got[0] - want[0]).max() <= 1e-12
        assert got[2][0] > 0
    tdm.device_status()


def test_noalloc_rejects_oversized_requests(tdm, cuda):
    import torch
    lib = tdm.lib()
    x = np.zeros((8, 3), np.float32)
    xd = torch.from_numpy(x).to(cuda)
    md = torch.tensor([8], dtype=torch.int32, device=cuda)
    rt = torch.zeros(12, dtype=torch.float64, device=cuda)
    inl = torch.zeros(8, dtype=torch.int32, device=cuda)
    info = torch.zeros(4, dtype=torch.int32, device=cuda)
    prm = tdm.RansacParams(1, MAX_TRIALS + 1, 0.05, 0, 50000)
    st = lib.tdm_ransac_noalloc(xd.data_ptr(), xd.data_ptr(), md.data_ptr(), 8, ctypes.byref(prm), rt.data_ptr(),
                                inl.data_ptr(), info.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert st == 1  # TDM_ERR_INVALID_ARG
    assert str(MAX_TRIALS) in lib.tdm_last_error().decode()
