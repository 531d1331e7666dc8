"""The C ABI library loads and exports every symbol include/*.h declares;
host-side argument and file checks run without a GPU."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(tdm_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def built(tdm):
    import __graft_entry__ as ge
    b = ge._load_file("tdm_gb300_build", os.path.join(ge.PKG_DIR, "build.py"))
    b.build()
    return tdm.lib()


def test_every_declared_symbol_is_exported(built, tdm):
    declared = _declared()
    assert len(declared) >= 35
    missing = [n for n in sorted(declared) if not hasattr(built, n)]
    assert not missing, missing
    assert set(tdm.EXPORTS) <= declared


def test_version_and_no_error(built, tdm):
    assert "sm_103a" in tdm.version()


def test_host_argument_checks(built, tdm):
    g = tdm.Grid()
    st = built.tdm_grid_from_points_host(None, 0, 0.01, 0.05, 15, ctypes.byref(g))
    assert st == 1  # INVALID_ARG
    assert "n <= 0" in built.tdm_last_error().decode()
    pts = np.zeros((3, 3), np.float32)
    st = built.tdm_grid_from_points_host(pts.ctypes.data, 3, 0.0, 0.05, 15, ctypes.byref(g))
    assert st == 1


def test_grid_host_matches_oracle(built, tdm, oracle):
    rng = np.random.default_rng(0)
    pts = rng.uniform(-1, 2, (5000, 3)).astype(np.float32)
    g = tdm.grid_from_points_host(pts)
    dim, origin = oracle.grid_setup(pts)
    assert tuple(g.dim) == tuple(dim.tolist())
    assert np.array_equal(np.array(g.origin, np.float32), origin)


def test_weight_file_errors(built, tdm, tmp_path):
    h = ctypes.c_void_p()
    st = built.tdm_net_create(str(tmp_path / "missing.marvin").encode(), 0, 1, ctypes.byref(h))
    assert st == 2  # IO: no retry loop, unlike Marvin's readTensors
    bad = tmp_path / "bad.marvin"
    bad.write_bytes(b"\x01\x04\x00\x00\x00\x05\x00\x00\x00conv")  # truncated record
    st = built.tdm_net_create(str(bad).encode(), 0, 1, ctypes.byref(h))
    assert st == 3  # FORMAT
    wrong = tmp_path / "wrong.marvin"
    wrong.write_bytes(b"\x09\x04\x00\x00\x00")  # int32 tensor type
    st = built.tdm_net_create(str(wrong).encode(), 0, 1, ctypes.byref(h))
    assert st == 3


def test_seeded_weights_file(built, tdm, oracle, tmp_path):
    p = str(tmp_path / "w.marvin")
    tdm.write_seeded_weights(p, 7)
    w = oracle.read_marvin(p)
    assert sorted(w) == sorted(n + s for n in oracle.NET_LAYERS for s in (".weight", ".bias"))
    for n, k, c, ks in zip(oracle.NET_LAYERS, oracle.NET_COUT, oracle.NET_CIN, oracle.NET_KS):
        a = w[n + ".weight"]
        assert a.shape == (k, c, ks, ks, ks)
        assert abs(a.std() / np.sqrt(2.0 / (c * ks ** 3)) - 1) < 0.05
        assert np.abs(w[n + ".bias"]).max() <= 0.05
    tdm.write_seeded_weights(str(tmp_path / "w2.marvin"), 7)
    assert open(p, "rb").read() == open(str(tmp_path / "w2.marvin"), "rb").read()


def test_grid_host_skips_nan_like_the_device_form(built, tdm):
    """The host bounds skip a NaN coordinate (fminf/fmaxf from +/-inf), the
    way the device min/max reduction does, even on the first point; an
    infinite coordinate is rejected."""
    rng = np.random.default_rng(1)
    pts = rng.uniform(-1, 2, (2000, 3)).astype(np.float32)
    bad = np.concatenate([np.array([[np.nan, 5.0, np.nan]], np.float32), pts])
    g, g_fin = tdm.grid_from_points_host(bad), tdm.grid_from_points_host(pts)
    # the NaN row's finite y = 5.0 widens the y extent, as on the device
    both = np.concatenate([np.array([[pts[0, 0], 5.0, pts[0, 2]]], np.float32), pts])
    g_both = tdm.grid_from_points_host(both)
    assert tuple(g.dim) == tuple(g_both.dim) and tuple(g.origin) == tuple(g_both.origin)
    assert g.dim[0] == g_fin.dim[0] and g.dim[2] == g_fin.dim[2]
    inf = np.concatenate([np.array([[np.inf, 0.0, 0.0]], np.float32), pts])
    st = built.tdm_grid_from_points_host(inf.ctypes.data, inf.shape[0], 0.01, 0.05, 15, ctypes.byref(tdm.Grid()))
    assert st == 1
