"""Pins the CPU oracle to the reference's own known answers (no GPU)."""
import glob
import json
import os

import numpy as np
import pytest

from conftest import golden, reference_path


def test_forsyth_ponce_recovers_sampledata(oracle):
    """demoEstimateRigidTransform.m: estimateRigidTransform(P2h, P1h) == T."""
    d = np.load(golden("sampledata.npz"))
    T = oracle.estimate_rigid_transform_fp(d["P2h"][:3], d["P1h"][:3])
    assert np.abs(T - d["T"]).max() < 1e-12
    assert np.abs(d["T"] @ d["P1h"] - d["P2h"]).max() < 1e-12


def test_kabsch_recovers_sampledata(oracle):
    """The product's Kabsch fit (x = R y + t) on the same known-answer data."""
    d = np.load(golden("sampledata.npz"))
    x = np.ascontiguousarray(d["P2h"][:3].T, np.float32)
    y = np.ascontiguousarray(d["P1h"][:3].T, np.float32)
    R, t = oracle.kabsch(x, y)
    assert np.abs(R - d["T"][:3, :3]).max() < 1e-6
    assert np.abs(t - d["T"][:3, 3]).max() < 1e-6
    # three-point fits (RANSAC's minimal sample) recover it too
    R3, t3 = oracle.kabsch(x, y, np.array([0, 100, 300], np.int32))
    assert np.abs(R3 - d["T"][:3, :3]).max() < 1e-5


def test_sample_cloud_geometry(oracle):
    """PLY reader and grid setup of core/demo.cu:69-124 on the reference's sample clouds."""
    ref = json.load(open(golden("sample_clouds.json")))
    assert ref["single-depth-1.ply"]["dim"] == [370, 253, 324]
    assert ref["single-depth-2.ply"]["dim"] == [299, 255, 263]
    for name, g in ref.items():
        path = reference_path("data/sample/3dmatch-demo", name)
        if not os.path.exists(path):
            pytest.skip("reference sample data not mounted")
        pts = oracle.read_ply(path)
        assert pts.shape[0] == g["n"]
        dim, origin = oracle.grid_setup(pts)
        assert dim.tolist() == g["dim"]
        assert np.array_equal(origin, np.array(g["origin"], np.float32))


def test_float_decode_quirk_counts(oracle):
    """core/demo.cu:32-34 decodes voxel indices in float32; voxels >= 2^24 of
    the sample grids land on the wrong centre (counts pinned in the fixture)."""
    ref = json.load(open(golden("sample_clouds.json")))
    for g in ref.values():
        dim = np.array(g["dim"], np.int32)
        assert oracle.count_misdecoded(dim, 1) == g["misdecoded_float32"]
        assert oracle.count_misdecoded(dim, 2) == g["misdecoded_fma"]
    assert ref["single-depth-1.ply"]["misdecoded_float32"] == 6776212
    assert ref["single-depth-2.ply"]["misdecoded_float32"] == 2037892
    # below 2^24 voxels every decode is exact
    assert oracle.count_misdecoded(np.array([256, 256, 255], np.int32), 1) == 0


def test_registration_metric_on_shipped_logs(oracle):
    """mrEvaluateRegistration.m restated: the shipped 3DMatch logs give the
    published mean recall / precision over the 8 real scenes."""
    dirs = sorted(d for d in glob.glob(reference_path("data/fragments/*-evaluation")) if "iclnuim" not in d)
    if not dirs:
        pytest.skip("reference fragments logs not mounted")
    R, P = [], []
    for d in dirs:
        r, p = oracle.evaluate_registration(oracle.read_log(d + "/3dmatch.log"), oracle.read_log(d + "/gt.log"),
                                            oracle.read_info(d + "/gt.info"))
        R.append(r)
        P.append(p)
    assert len(R) == 8
    assert abs(np.mean(R) - 0.6678) < 5e-5
    assert abs(np.mean(P) - 0.4009) < 5e-5
