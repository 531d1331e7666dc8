"""Product-side benchmark bookkeeping (tdm_gb300.evaluation): log I/O, the
writeLog.m filter, mrEvaluateRegistration.m and getError.m, pinned to the
numbers the reference's shipped logs give."""
import glob
import os

import numpy as np
import pytest

from conftest import REFERENCE


@pytest.fixture(scope="module")
def ev():
    import __graft_entry__ as ge
    ge.load()
    from tdm_gb300 import evaluation
    return evaluation


def test_log_roundtrip_and_filter(ev, tmp_path):
    rng = np.random.default_rng(1)
    results = []
    for i in range(4):
        for j in range(i + 1, 4):
            rt = np.eye(4)
            rt[:3, 3] = rng.normal(size=3)
            results.append((i, j, rt, rng.uniform(0, 1)))
    recs = ev.log_records(results, 4)
    assert [(i, j) for i, j, _, _ in recs] == [(i, j) for i, j, _, r in results if r > 0.30]
    ev.write_log(tmp_path / "x.log", recs)
    back = ev.read_log(tmp_path / "x.log")
    assert [(i, j, n) for i, j, n, _ in back] == [(i, j, n) for i, j, n, _ in recs]
    for (_, _, _, a), (_, _, _, b) in zip(back, recs):
        assert np.allclose(a, b, atol=1e-10)


def test_registration_metric_on_shipped_logs(ev):
    """The shipped 3DMatch logs give the published mean recall / precision."""
    dirs = sorted(d for d in glob.glob(os.path.join(REFERENCE, "data/fragments/*-evaluation")) if "iclnuim" not in d)
    if not dirs:
        pytest.skip("reference fragment logs not mounted")
    R, P = [], []
    for d in dirs:
        r, p = ev.evaluate_registration(ev.read_log(d + "/3dmatch.log"), ev.read_log(d + "/gt.log"),
                                        ev.read_info(d + "/gt.info"))
        R.append(r)
        P.append(p)
    assert len(R) == 8
    assert abs(np.mean(R) - 0.6678) < 5e-5 and abs(np.mean(P) - 0.4009) < 5e-5


def test_keypoint_matching_error_on_shipped_log(ev):
    """getError.m on the shipped 3DMatch distances and validation labels."""
    d = os.path.join(REFERENCE, "evaluation/keypoint-matching")
    if not os.path.exists(os.path.join(d, "validation-set-gt.log")):
        pytest.skip("reference keypoint-matching logs not mounted")
    err = ev.fpr_at_95_recall(ev.read_distance_log(os.path.join(d, "3dmatch.log")),
                              ev.read_distance_log(os.path.join(d, "validation-set-gt.log")))
    assert abs(err - 0.3517) < 5e-5, err


def test_fpr_definition(ev):
    """Perfectly separated distances: no false positive at 95 % recall."""
    d = np.concatenate([np.linspace(0.0, 1.0, 100), np.linspace(2.0, 3.0, 100)])
    m = np.concatenate([np.ones(100), np.zeros(100)])
    assert ev.fpr_at_95_recall(d, m) == 0.0


def test_info_roundtrip_and_information(ev, tmp_path):
    q = np.random.default_rng(3).normal(size=(50, 3))
    M = ev.gt_information(q)
    assert np.allclose(M, M.T) and np.allclose(M[:3, :3], 50 * np.eye(3))
    ev.write_info(tmp_path / "g.info", [(0, 2, 5, M)])
    (i, j, n, back), = ev.read_info(tmp_path / "g.info")
    assert (i, j, n) == (0, 2, 5) and np.allclose(back, M, rtol=1e-7)
    # a result equal to the ground truth is correct; one 0.5 m off is not
    gt = [(0, 2, 5, np.eye(4))]
    off = np.eye(4)
    off[0, 3] = 0.5
    assert ev.evaluate_registration([(0, 2, 5, np.eye(4))], gt, [(0, 2, 5, M)]) == (1.0, 1.0)
    assert ev.evaluate_registration([(0, 2, 5, off)], gt, [(0, 2, 5, M)]) == (0.0, 0.0)
