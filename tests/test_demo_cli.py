"""The drop-in `demo <cloud.ply> <out_prefix>` binary (core/demo.cu's CLI):
exit codes of its input checks (no GPU needed), and on a GPU the files it
writes, byte for byte equal to the library's results."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DEMO = os.path.join(ROOT, "3dmatch-toolbox_gb300", "bin", "demo")


def _write_ply(path, pts, count_line=True):
    with open(path, "wb") as f:
        hdr = ["ply", "format binary_little_endian 1.0",
               "element vertex %d" % pts.shape[0] if count_line else "comment no count",
               "property float x", "property float y", "property float z", "end_header"]
        f.write(("\n".join(hdr) + "\n").encode())
        f.write(np.ascontiguousarray(pts, "<f4").tobytes())


def _need_demo():
    if not os.path.exists(DEMO):
        pytest.skip("bin/demo not built")


def test_missing_cloud_exits_minus_one(tmp_path):
    _need_demo()
    r = subprocess.run([DEMO, str(tmp_path / "absent.ply"), str(tmp_path / "out")], capture_output=True)
    assert r.returncode == 255  # -1, core/demo.cu:71-74
    assert b"not found" in r.stderr


def test_missing_vertex_count_exits_zero(tmp_path):
    _need_demo()
    p = tmp_path / "nocount.ply"
    _write_ply(p, np.zeros((4, 3), np.float32), count_line=False)
    r = subprocess.run([DEMO, str(p), str(tmp_path / "out")], capture_output=True)
    assert r.returncode == 0  # core/demo.cu:84-87
    assert not (tmp_path / "out.keypts.bin").exists()


def test_demo_reads_the_reference_sample_clouds():
    """The drop-in's own C++ PLY reader and host grid setup on the
    reference's sample clouds (data/sample/3dmatch-demo, read in place where
    the reference tree is mounted): vertex count, first and last point and
    grid geometry equal the golden values derived by the oracle
    (core/demo.cu:69-124)."""
    import json
    from conftest import golden, reference_path
    _need_demo()
    want = json.load(open(golden("sample_clouds.json")))
    for name, g in want.items():
        path = reference_path("data/sample/3dmatch-demo", name)
        if not os.path.exists(path):
            pytest.skip("reference sample clouds not mounted")
        r = subprocess.run([DEMO, path, "/nonexistent/out", "--info"], capture_output=True)
        assert r.returncode == 0, r.stderr.decode()
        out = r.stdout.decode().split("\n")
        assert "Loaded point cloud with %d points!" % g["n"] in out
        tok = next(l for l in out if l.startswith("points ")).split()
        assert int(tok[1]) == g["n"]
        assert np.array_equal(np.float32(tok[3:6]), np.float32(g["first"]))
        assert np.array_equal(np.float32(tok[7:10]), np.float32(g["last"]))
        tok = next(l for l in out if l.startswith("grid ")).split()
        assert [int(t) for t in tok[1:4]] == g["dim"]
        assert np.array_equal(np.float32(tok[5:8]), np.float32(g["origin"]))


@pytest.mark.gpu
def test_demo_files_equal_library(tdm, scene, cuda, tmp_path):
    import torch
    _need_demo()
    pts = scene.fragment(20264000, n_points=60_000)
    _write_ply(tmp_path / "cloud.ply", pts)
    k, seed = 120, 11
    r = subprocess.run([DEMO, "cloud.ply", "out", "--seeded-weights", "7", "--seed", str(seed), "--keypoints", str(k),
                        "--tdf-out"], cwd=tmp_path, capture_output=True)
    assert r.returncode == 0, r.stderr.decode()
    kp_file = np.fromfile(tmp_path / "out.keypts.bin", "<f4")
    desc_file = np.fromfile(tmp_path / "out.desc.3dmatch.bin", "<f4")
    tdf_file = np.fromfile(tmp_path / "tdf.bin", "<f4")
    assert kp_file[0] == k and kp_file.size == 1 + 3 * k
    assert desc_file[0] == k and desc_file[1] == 512 and desc_file.size == 2 + 512 * k
    # the same steps through the library
    g = tdm.grid_from_points_host(pts)
    pd = torch.from_numpy(pts).to(cuda)
    tdf = tdm.tdf(pd, g)
    kp, kg = tdm.keypoints(pd, tdm.keypoint_indices(seed, pts.shape[0], k, device=cuda), g)
    net = tdm.Net(marvin_path=str(tmp_path / "out.seeded-weights.marvin"), precision="fp32")
    desc = net.forward(tdm.gather(tdf, g, kg))
    assert np.array_equal(kp_file[1:].reshape(k, 3), kp.cpu().numpy())
    assert np.array_equal(desc_file[2:].reshape(k, 512), desc.cpu().numpy())
    assert np.array_equal(tdf_file[:3], np.array(g.dim, np.float32))
    assert np.array_equal(tdf_file[8:], tdf.cpu().numpy())


DESCRIPTORS = os.path.join(ROOT, "3dmatch-toolbox_gb300", "bin", "descriptors")


@pytest.mark.gpu
def test_descriptors_volume_form(tdm, scene, cuda, tmp_path):
    """get3DMatchDescriptors.cu (keypoint matching): volumes in, feat.bin out,
    whole batches of 50 only unless --all."""
    import torch
    if not os.path.exists(DESCRIPTORS):
        pytest.skip("bin/descriptors not built")
    pts = scene.fragment(20264100, n_points=60_000)
    g = tdm.grid_from_points_host(pts)
    pd = torch.from_numpy(pts).to(cuda)
    _, kg = tdm.keypoints(pd, tdm.keypoint_indices(5, pts.shape[0], 120, device=cuda), g)
    patches = tdm.gather(tdm.tdf(pd, g), g, kg)
    with open(tmp_path / "vol.bin", "wb") as f:
        f.write(np.array([120, 30, 30, 30], "<f4").tobytes())
        f.write(patches.cpu().numpy().astype("<f4").tobytes())
    r = subprocess.run([DESCRIPTORS, "vol.bin", "--seeded-weights", "3"], cwd=tmp_path, capture_output=True)
    assert r.returncode == 0, r.stderr.decode()
    feat = np.fromfile(tmp_path / "feat.bin", "<f4")
    assert np.array_equal(feat[:5], np.array([120, 512, 1, 1, 1], np.float32))
    assert feat.size == 5 + 100 * 512  # two whole batches
    net = tdm.Net(marvin_path=str(tmp_path / "vol.bin.seeded-weights.marvin"), precision="fp32")
    want = net.forward(patches).cpu().numpy()
    assert np.array_equal(feat[5:].reshape(100, 512), want[:100])
    r = subprocess.run([DESCRIPTORS, "vol.bin", "--seeded-weights", "3", "--all", "--out", "all.bin"], cwd=tmp_path,
                       capture_output=True)
    assert r.returncode == 0
    assert np.array_equal(np.fromfile(tmp_path / "all.bin", "<f4")[5:].reshape(120, 512), want)


@pytest.mark.gpu
def test_descriptors_grid_form(tdm, scene, cuda, tmp_path):
    """get3DMatchDescriptors.cu (shape2pose): a TDF grid and keypoint grid
    coordinates in, <name>.3dmatch.descriptors.bin out."""
    import torch
    if not os.path.exists(DESCRIPTORS):
        pytest.skip("bin/descriptors not built")
    pts = scene.fragment(20264200, n_points=60_000)
    g = tdm.grid_from_points_host(pts)
    pd = torch.from_numpy(pts).to(cuda)
    tdf = tdm.tdf(pd, g)
    _, kg = tdm.keypoints(pd, tdm.keypoint_indices(6, pts.shape[0], 60, device=cuda), g)
    with open(tmp_path / "obj.TDF.bin", "wb") as f:
        f.write(np.array(list(g.dim), "<f4").tobytes())
        f.write(tdf.cpu().numpy().astype("<f4").tobytes())
    kgf = kg.cpu().numpy().astype(np.float32) + np.float32(0.25)  # rounded back by the tool
    with open(tmp_path / "obj.keypoints.bin", "wb") as f:
        f.write(np.array([60], "<f4").tobytes())
        f.write(kgf.astype("<f4").tobytes())
    r = subprocess.run([DESCRIPTORS, "obj.TDF.bin", "obj.keypoints.bin", "--seeded-weights", "4"], cwd=tmp_path,
                       capture_output=True)
    assert r.returncode == 0, r.stderr.decode()
    out = np.fromfile(tmp_path / "obj.keypoints.3dmatch.descriptors.bin", "<f4")
    assert out[0] == 60 and out[1] == 512 and out.size == 2 + 50 * 512
    net = tdm.Net(marvin_path=str(tmp_path / "obj.keypoints.bin.seeded-weights.marvin"), precision="fp32")
    want = net.forward(tdm.gather(tdf, g, kg)).cpu().numpy()
    assert np.array_equal(out[2:].reshape(50, 512), want[:50])


FUSE = os.path.join(ROOT, "3dmatch-toolbox_gb300", "bin", "fuse")


def _png16(path, img, first_filter):
    """16-bit grey PNG; row filters cycle through None, Sub, Up, Average, Paeth."""
    import struct
    import zlib
    h, w = img.shape
    data = np.ascontiguousarray(img.astype(">u2")).view(np.uint8).reshape(h, 2 * w).astype(np.int32)
    prev = np.zeros(2 * w, np.int32)
    rows = []
    for r in range(h):
        cur = data[r]
        left = np.concatenate([[0, 0], cur[:-2]])
        upleft = np.concatenate([[0, 0], prev[:-2]])
        t = (first_filter + r) % 5
        if t == 0:
            f = cur
        elif t == 1:
            f = cur - left
        elif t == 2:
            f = cur - prev
        elif t == 3:
            f = cur - (left + prev) // 2
        else:
            p = left + prev - upleft
            pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - upleft)
            f = cur - np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
        rows.append(bytes([t]) + (f % 256).astype(np.uint8).tobytes())
        prev = cur

    def chunk(kind, payload):
        return struct.pack(">I", len(payload)) + kind + payload + struct.pack(">I", zlib.crc32(kind + payload))

    with open(path, "wb") as fh:
        fh.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 16, 0, 0, 0, 0)) +
                 chunk(b"IDAT", zlib.compress(b"".join(rows))) + chunk(b"IEND", b""))


@pytest.mark.gpu
def test_fuse_cli_equals_library(tdm, scene, cuda, tmp_path):
    """depth-fusion/demo.cu's CLI: PNG depth frames and pose files in, the
    tsdf.ply surface of the library's TSDF out, bit for bit."""
    import torch
    if not os.path.exists(FUSE):
        pytest.skip("bin/fuse not built")
    frames, poses = scene.depth_sequence(20264300, n_frames=6)
    poses = np.asarray(poses, np.float32).copy()
    poses[0] = np.eye(4, dtype=np.float32)  # an exact identity base pose: cam2base = the pose files
    d = tmp_path / "frames"
    d.mkdir()
    for i in range(6):
        _png16(d / ("frame-%06d.depth.png" % i), frames[i], i)
        np.savetxt(d / ("frame-%06d.pose.txt" % i), poses[i].reshape(4, 4), fmt="%.9g")
    np.savetxt(tmp_path / "K.txt", np.array([[585, 0, 320], [0, 585, 240], [0, 0, 1]], np.float32), fmt="%.9g")
    args = ["K.txt", "frames", "0", "0", "6", "-1.536", "-1.536", "0.5", "0.012", "0.06", "--dims", "256", "256", "256"]
    r = subprocess.run([FUSE] + args, cwd=tmp_path, capture_output=True)
    assert r.returncode == 0, r.stderr.decode()
    raw = open(tmp_path / "tsdf.ply", "rb").read()
    hdr, body = raw.split(b"end_header\n", 1)
    n = int([ln for ln in hdr.decode().splitlines() if ln.startswith("element vertex")][0].split()[2])
    got = np.frombuffer(body, "<f4").reshape(n, 3)
    # the same fusion through the library
    dim, origin = [256, 256, 256], [np.float32(-1.536), np.float32(-1.536), np.float32(0.5)]
    mm = torch.from_numpy(frames.astype(np.uint16).view(np.int16)).to(cuda)
    depth = torch.empty(frames.shape, dtype=torch.float32, device=cuda)
    ts = torch.empty(256 ** 3, dtype=torch.float32, device=cuda)
    wt = torch.empty(256 ** 3, dtype=torch.float32, device=cuda)
    tdm.depth_from_mm(mm, depth)
    tdm.tsdf_init(ts, wt, dim)
    tdm.tsdf_integrate(ts, wt, dim, origin, np.float32(0.012), np.float32(0.06), depth,
                       np.array([585, 0, 320, 0, 585, 240, 0, 0, 1], np.float32), poses)
    pts, cnt = tdm.tsdf_extract(ts, wt, dim, origin, np.float32(0.012))
    want = pts[:int(cnt.item())].cpu().numpy()
    assert n == want.shape[0] and n > 1000
    assert np.array_equal(got, want)
