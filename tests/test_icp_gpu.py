"""ICP refinement (the step register2Fragments.m:70-78 leaves commented out):
one iteration equal to the oracle's FP64 restatement, bit-identical repeats,
recovery of a rigid motion of a cloud, a fixed point at an exact alignment.
(Trimmed point-to-point ICP with the reference's 30 % inlier ratio slides
along the planes of the synthetic rooms; these tests fix the algorithm, not
its basin of attraction.)"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rot(axis, deg):
    axis = np.asarray(axis, float) / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    a = np.radians(deg)
    return np.eye(3) + np.sin(a) * K + (1 - np.cos(a)) * K @ K


def _errors(T, G):
    dR = G[:3, :3].T @ T[:3, :3]
    ang = np.degrees(np.arccos(np.clip((np.trace(dR) - 1) / 2, -1, 1)))
    return ang, np.linalg.norm(T[:3, 3] - G[:3, 3])


@pytest.fixture(scope="module")
def pair(scene):
    a, b, gt = scene.fragment_pair(20268000, n_points=80_000)
    return a, b, np.asarray(gt, np.float64)


def _init(gt):
    init = gt.copy()
    init[:3, :3] = _rot([1, 2, 3], 2.0) @ gt[:3, :3]
    init[:3, 3] += np.array([0.02, -0.015, 0.01])
    return init


@pytest.mark.parametrize("ratio", [0.3, 1.0])
def test_one_iteration_equals_oracle(tdm, oracle, cuda, pair, ratio):
    import torch
    a, b, gt = pair
    init = _init(gt)
    T, res = tdm.icp(torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda), init, inlier_ratio=ratio,
                     max_iterations=1)
    want = oracle.icp(a, b, init, inlier_ratio=ratio, iterations=1)
    assert res.iterations == 1
    ang, tr = _errors(T, want)
    assert ang < 1e-3 and tr < 1e-5, (ang, tr)


def test_repeats_are_bit_identical(tdm, cuda, pair):
    import torch
    a, b, gt = pair
    da, db = torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda)
    T1, r1 = tdm.icp(da, db, _init(gt))
    T2, r2 = tdm.icp(da, db, _init(gt))
    assert np.array_equal(T1, T2) and r1.iterations == r2.iterations and r1.rmse == r2.rmse


def test_recovers_rigid_motion(tdm, cuda, pair):
    """moving = a rigidly moved copy of fixed: ICP from the identity recovers
    the inverse motion."""
    import torch
    a = pair[0]
    R, t = _rot([0.3, -1.0, 0.5], 1.5), np.array([0.012, -0.008, 0.015])
    moving = (a.astype(np.float64) @ R.T + t).astype(np.float32)
    G = np.eye(4)
    G[:3, :3] = R.T
    G[:3, 3] = -R.T @ t
    T, res = tdm.icp(torch.from_numpy(a).to(cuda), torch.from_numpy(moving).to(cuda), np.eye(4), inlier_ratio=1.0,
                     max_iterations=100)
    ang, tr = _errors(T, G)
    # the 1 cm grid averages of a moved copy are not the moved averages: mm-level residual
    assert ang < 0.05 and tr < 2e-3, (ang, tr, res.iterations)
    assert res.converged == 1


def test_exact_alignment_stays(tdm, cuda, pair):
    import torch
    da = torch.from_numpy(pair[0]).to(cuda)
    T, res = tdm.icp(da, da, np.eye(4))
    assert np.abs(T - np.eye(4)).max() < 1e-6
    assert res.converged == 1


def test_bad_input(tdm, cuda, pair):
    import torch
    far = torch.full((10, 3), 1.0e6, dtype=torch.float32, device=cuda)
    with pytest.raises(tdm.TdmError):
        tdm.icp(torch.from_numpy(pair[0]).to(cuda), far, np.eye(4))
    tdm.device_status()
