"""GPU surface overlap (register2Fragments.m:90-97) against the oracle's
brute force: counts bit-exact (same float arithmetic, strict d2 < r^2)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rt(rng, ang=0.4, t=0.3):
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
    return np.concatenate([R, rng.normal(size=(3, 1)) * t], 1)


@pytest.mark.parametrize("na,nb", [(1, 1), (3000, 2000), (20000, 25000)])
def test_random_clouds(tdm, oracle, cuda, na, nb):
    import torch
    rng = np.random.default_rng(na + nb)
    a = rng.uniform(-1, 1, (na, 3)).astype(np.float32)
    b = rng.uniform(-1, 1, (nb, 3)).astype(np.float32)
    rt = _rt(rng)
    got = tdm.overlap(torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda), rt, 0.05)
    assert got == oracle.overlap(a, b, rt, 0.05)


def test_registered_pair(tdm, oracle, scene, cuda):
    """A synthetic pair under its ground-truth transform overlaps far more
    than under a perturbed one; both counts equal the oracle's."""
    import torch
    a, b, gt = scene.fragment_pair(20265000, n_points=20_000)
    da, db = torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda)
    good = tdm.overlap(da, db, np.asarray(gt)[:3], 0.05)
    assert good == oracle.overlap(a, b, np.asarray(gt)[:3], 0.05)
    bad_rt = np.asarray(gt, np.float64)[:3].copy()
    bad_rt[:, 3] += 0.2
    bad = tdm.overlap(da, db, bad_rt, 0.05)
    assert bad == oracle.overlap(a, b, bad_rt, 0.05)
    assert good[0] / a.shape[0] > 0.3 and good[0] > bad[0]


def test_boundary_and_limits(tdm, cuda):
    import torch
    r = np.float32(0.05)
    a = np.array([[0, 0, 0], [1, 1, 1]], np.float32)
    b = np.array([[r, 0, 0], [1, 1, 1 + np.float32(0.049)]], np.float32)  # exactly r: not counted (strict)
    got = tdm.overlap(torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda), np.eye(4)[:3], float(r))
    assert got == (1, 1)
    far = np.array([[1.0e5, 0, 0]], np.float32)
    with pytest.raises(tdm.TdmError, match="grid cells"):
        tdm.overlap(torch.from_numpy(far).to(cuda), torch.from_numpy(b).to(cuda), np.eye(4)[:3], 0.05)
    tdm.device_status()
