"""GPU parity of the descriptor net against the oracle.

Tolerances: FP32 form <= 1e-4 relative L2 against the FP32 oracle forward;
BF16 tensor-core form <= 1e-2 relative L2 against the FP64 oracle forward.
Each tensor-core layer (BF16 and FP8 forms) <= 1e-3 against the float64
restatement of its operand and storage rounding applied to its own GPU input,
with at most 1 % of stored values one rounding step apart.  The FP8 form's
distance from the exact net (~8e-2) equals that of its restatement and is
outside the 1e-2 descriptor tolerance.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RESPONSES = ["conv1", "conv2", "pool1", "conv3", "conv4", "conv5", "conv6", "conv7", "conv8", "feat"]
FP8_LAYERS = (2, 3, 4, 5, 6, 7)  # conv3..conv8 take E4M3 operands in the FP8 form
# One tensor-core layer against the float64 restatement of its own operand and
# storage rounding, on the GPU's own stored input: only the FP32 sums differ.
LAYER_TOL = 1e-3
LAYER_DIFFER = 1e-2  # fraction of stored values allowed one rounding step apart


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def weights(oracle):
    return oracle.he_normal_weights(20260001)


@pytest.fixture(scope="module")
def patches(tdm, oracle, scene, cuda):
    """Real TDF patches of a synthetic fragment (the demo path)."""
    import torch
    pts = scene.fragment(20260002)
    g = tdm.grid_from_points_host(pts)
    pd = torch.from_numpy(pts).to(cuda)
    tdf = tdm.tdf(pd, g)
    idx = tdm.keypoint_indices(3, pts.shape[0], 12, device=cuda)
    _, kg = tdm.keypoints(pd, idx, g)
    return tdm.gather(tdf, g, kg)


def _oracle_responses(oracle, p, w):
    """Per-layer float64 responses, channels-last, via the oracle's conv loops."""
    out = {}
    x = p.reshape(-1, 30, 30, 30, 1).astype(np.float64)
    B = x.shape[0]
    D, C = 30, 1
    for i, n in enumerate(oracle.NET_LAYERS):
        K, ks = oracle.NET_COUT[i], oracle.NET_KS[i]
        Do = D - ks + 1
        y = np.zeros((B, Do, Do, Do, K))
        lib = oracle.lib()
        xin = np.ascontiguousarray(x)
        wt = np.ascontiguousarray(w[n + ".weight"], np.float32)
        bt = np.ascontiguousarray(w[n + ".bias"].reshape(-1), np.float32)
        lib.orc_conv3d_f64(xin.ctypes.data, B, D, C, wt.ctypes.data, bt.ctypes.data, K, ks, 1 if i < 8 else 0,
                           y.ctypes.data)
        out[n] = y
        x, D, C = y, Do, K
        if i == 1:
            Dp = D // 2
            z = np.zeros((B, Dp, Dp, Dp, C))
            lib.orc_pool_f64(np.ascontiguousarray(x).ctypes.data, B, D, C, z.ctypes.data)
            out["pool1"] = z
            x, D = z, Dp
    return out


@pytest.fixture(scope="module")
def oracle_resp(oracle, patches, weights):
    return _oracle_responses(oracle, patches.cpu().numpy()[:4], weights)


def test_fp32_descriptors(tdm, oracle, weights, patches):
    net = tdm.Net(weights, precision="fp32")
    got = net.forward(patches).cpu().numpy()
    want = oracle.net_forward(patches.cpu().numpy(), weights)
    assert rel_l2(got, want) <= 1e-4
    want64 = oracle.net_forward(patches.cpu().numpy(), weights, f64=True)
    assert rel_l2(got, want64) <= 1e-4
    tdm.device_status()


@pytest.mark.parametrize("name", RESPONSES)
def test_fp32_responses(tdm, weights, patches, oracle_resp, name):
    net = tdm.Net(weights, precision="fp32")
    got = net.response(name, patches[:4]).cpu().numpy()
    assert rel_l2(got, oracle_resp[name]) <= 1e-5, name


@pytest.mark.parametrize("name", RESPONSES)
def test_bf16_responses(tdm, weights, patches, oracle_resp, name):
    net = tdm.Net(weights, precision="bf16")
    got = net.response(name, patches[:4]).cpu().numpy()
    assert rel_l2(got, oracle_resp[name]) <= 1e-2, name
    tdm.device_status()


def test_bf16_descriptors(tdm, oracle, weights, patches):
    net = tdm.Net(weights, precision="bf16")
    got = net.forward(patches).cpu().numpy()
    want64 = oracle.net_forward(patches.cpu().numpy(), weights, f64=True)
    assert rel_l2(got, want64) <= 1e-2
    tdm.device_status()


def test_bf16_batch_independence(tdm, weights, patches):
    """A patch's descriptor does not depend on its batch neighbours or chunking."""
    import torch
    net = tdm.Net(weights, precision="bf16")
    full = net.forward(patches).cpu().numpy()
    one = net.forward(patches[5:6].contiguous()).cpu().numpy()
    assert np.array_equal(full[5:6], one)
    net.set_max_batch(5)
    chunked = net.forward(patches).cpu().numpy()
    assert np.array_equal(full, chunked)


def test_marvin_file_path(tdm, oracle, patches, tmp_path):
    """Weights written by the library load by name like Marvin's loadWeights."""
    p = str(tmp_path / "seeded.marvin")
    tdm.write_seeded_weights(p, 99)
    w = oracle.read_marvin(p)
    assert w["conv1.weight"].shape == (64, 1, 3, 3, 3) and w["feat.bias"].shape == (1, 512, 1, 1, 1)
    net = tdm.Net(marvin_path=p, precision="fp32")
    got = net.forward(patches[:3]).cpu().numpy()
    want = oracle.net_forward(patches[:3].cpu().numpy(), w)
    assert rel_l2(got, want) <= 1e-4




@pytest.fixture(scope="module")
def fp8_net(tdm, weights, patches):
    net = tdm.Net(weights, precision="fp8")
    net.calibrate(patches[:4].contiguous())  # the oracle responses cover these four
    return net


def test_fp8_requires_calibration(tdm, weights, patches):
    net = tdm.Net(weights, precision="fp8")
    with pytest.raises(tdm.TdmError, match="calibrate"):
        net.forward(patches)


def test_fp8_scales(fp8_net, oracle_resp):
    sc = fp8_net.act_scales()
    # scale of layer l's input = max of layer l-1's response / 448 (responses of the BF16 form)
    for l, name in zip(range(2, 8), ["conv2", "conv3", "conv4", "conv5", "conv6", "conv7"]):
        assert sc[l] > 0
        assert abs(sc[l] * 448 / oracle_resp[name].max() - 1) < 0.05, name


# Stored formats of each layer's input and output in the tensor-core forms:
# (name, input response, E4M3 input, stored output) per layer index.
LAYERS = [("conv1", None), ("conv2", "conv1"), ("conv3", "pool1"), ("conv4", "conv3"), ("conv5", "conv4"),
          ("conv6", "conv5"), ("conv7", "conv6"), ("conv8", "conv7"), ("feat", "conv8")]


def _formats(precision, l, scales):
    """(E4M3 input, input scale, output kind, output scale) of layer l."""
    fp8 = precision == "fp8"
    fin = fp8 and l in FP8_LAYERS
    nxt = l + 1
    out = "f32" if l == 8 else ("e4m3" if fp8 and nxt in FP8_LAYERS else "bf16")
    return fin, (scales[l] if fin else 1.0), out, (scales[nxt] if out == "e4m3" else 1.0)


def _check_layers(tdm, oracle, net, precision, weights, batch, rows):
    """Every layer of `net`, run by the GPU on `batch`, against the float64
    restatement of that one layer applied to the GPU's own stored input (for
    the patches `rows`): only the FP32 sums differ, so a stored rounding lands
    differently on a few elements at most."""
    scales = net.act_scales() if precision == "fp8" else np.ones(9, np.float32)
    report = {}
    for l, (name, src) in enumerate(LAYERS):
        x = (batch[rows].cpu().numpy().reshape(-1, 30, 30, 30, 1) if src is None
             else net.response(src, batch)[rows].cpu().numpy()).astype(np.float64)
        got = net.response(name, batch)[rows].cpu().numpy()
        fin, sin, out, sout = _formats(precision, l, scales)
        want = oracle.net_layer_quantized(x, weights, l, fin, sin, out, sout)
        err = rel_l2(got, want)
        # stored (rounded) outputs: the fraction one rounding step apart;
        # feat's float output has no rounding step, only the FP32 sums
        differ = float(np.mean(got != want.astype(np.float32))) if out != "f32" else 0.0
        report[name] = (float("%.3g" % err), float("%.3g" % differ))
        assert err <= LAYER_TOL and differ <= LAYER_DIFFER, (name, err, differ)
    print(precision, "per layer (rel-L2, fraction of stored values that differ):", report)


@pytest.mark.parametrize("precision", ["bf16", "fp8"])
def test_layers_on_their_own_inputs(tdm, oracle, weights, patches, precision):
    net = tdm.Net(weights, precision=precision)
    if precision == "fp8":
        net.calibrate(patches[:4].contiguous())
    _check_layers(tdm, oracle, net, precision, weights, patches[:4].contiguous(), slice(0, 4))
    net.close()
    tdm.device_status()


def test_fp8_descriptors(tdm, oracle, fp8_net, weights, patches):
    """The FP8 form's distance from the exact FP64 net is what E4M3 rounding
    of conv3..conv8 gives (the float64 restatement of the same rounding lands
    at the same distance): ~8e-2, outside the 1e-2 descriptor tolerance that
    the BF16 form meets."""
    p = patches.cpu().numpy()
    got = fp8_net.forward(patches).cpu().numpy()
    want64 = oracle.net_forward(p, weights, f64=True)
    emu = oracle.net_forward_quantized(p, weights, FP8_LAYERS, fp8_net.act_scales())
    err, err_emu = rel_l2(got, want64), rel_l2(emu, want64)
    print("fp8 descriptor rel-L2 vs FP64: %.4g (restatement of its rounding: %.4g)" % (err, err_emu))
    assert abs(err - err_emu) <= 0.25 * err_emu
    tdm.device_status()


@pytest.fixture(scope="module")
def chunk_patches(tdm, scene, cuda):
    """2,048 pipeline patches: one full internal chunk of the net, the launch
    size the pair bench times (persistent tile loops with many tiles per CTA,
    conv8's four-way split K)."""
    import torch
    pts = scene.fragment(20260004)
    g = tdm.grid_from_points_host(pts)
    pd = torch.from_numpy(pts).to(cuda)
    tdf = tdm.tdf(pd, g)
    idx = tdm.keypoint_indices(11, pts.shape[0], 2048, device=cuda)
    _, kg = tdm.keypoints(pd, idx, g)
    return tdm.gather(tdf, g, kg)


# 16 patches spread over the chunk: both ends, tile and sub-tile edges, the rest seeded
SAMPLED = sorted(set([0, 1, 127, 128, 1023, 1024, 2046, 2047] +
                     np.random.default_rng(5).choice(2048, 8, replace=False).tolist()))


@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp8"])
def test_descriptors_at_the_timed_launch_size(tdm, oracle, weights, chunk_patches, precision):
    net = tdm.Net(weights, precision=precision)
    if precision == "fp8":
        net.calibrate(chunk_patches[:256].contiguous())
    got = net.forward(chunk_patches).cpu().numpy()[SAMPLED]
    p = chunk_patches.cpu().numpy()[SAMPLED]
    want64 = oracle.net_forward(p, weights, f64=True)
    err = rel_l2(got, want64)
    print(precision, "2048-patch launch, 16 sampled descriptors, rel-L2 vs FP64: %.4g" % err)
    if precision == "fp32":
        assert err <= 1e-4
    elif precision == "bf16":
        assert err <= 1e-2
    else:
        emu = rel_l2(oracle.net_forward_quantized(p, weights, FP8_LAYERS, net.act_scales()), want64)
        assert abs(err - emu) <= 0.25 * emu
    net.close()
    tdm.device_status()


@pytest.mark.parametrize("precision", ["bf16", "fp8"])
def test_layers_at_the_timed_launch_size(tdm, oracle, weights, chunk_patches, precision):
    """Each layer of a 2,048-patch forward (every tile form and split the
    bench's launches use) against the one-layer restatement on its own
    inputs, for the 16 sampled patches."""
    net = tdm.Net(weights, precision=precision)
    if precision == "fp8":
        net.calibrate(chunk_patches[:256].contiguous())
    _check_layers(tdm, oracle, net, precision, weights, chunk_patches, SAMPLED)
    net.close()
    tdm.device_status()


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_fresh_nets_on_nonblocking_streams(tdm, weights, patches, precision):
    """The first forward of new nets, issued at once from several threads on
    streams that do not wait for the legacy stream, equals a settled forward
    (workspace zeroing and weight uploads are ordered before first use)."""
    import threading
    import torch
    ref = tdm.Net(weights, precision=precision).forward(patches)
    torch.cuda.synchronize()
    nets = [tdm.Net(weights, precision=precision) for _ in range(4)]
    outs = [None] * 4

    def run(t):
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            outs[t] = nets[t].forward(patches, stream=s)
            s.synchronize()

    th = [threading.Thread(target=run, args=(t,)) for t in range(4)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    for t in range(4):
        assert torch.equal(outs[t], ref), t


@pytest.mark.parametrize("precision", ["bf16", "fp8"])
@pytest.mark.parametrize("nb", [1, 3, 6])
def test_fused_x_pool_same_bits(tdm, weights, patches, precision, nb):
    """conv2's epilogue takes the pool's x-, z- and (within a CTA half) y-pair
    max, and a small pass the y pairs that cross halves; pool1 equals the
    2x2x2 max of the unfused conv2 response bit for bit (max commutes with the
    rounding).  One patch splits the z walk into short units."""
    net = tdm.Net(weights, precision=precision)
    if precision == "fp8":
        net.calibrate(patches)
    b = patches[:nb].contiguous()
    c2 = net.response("conv2", b).cpu().numpy()   # [b, 26, 26, 26, 64], unfused epilogue
    p1 = net.response("pool1", b).cpu().numpy()   # [b, 13, 13, 13, 64], fused pair maxima
    want = c2.reshape(nb, 13, 2, 13, 2, 13, 2, 64).max(axis=(2, 4, 6))
    assert np.array_equal(p1, want)
    tdm.device_status()


def test_half_typed_marvin_file(tdm, oracle, weights, patches, tmp_path):
    """A .marvin file whose records are half (type id 0), as Marvin writes
    weights when StorageT is half (core/marvin.hpp:2634-2705, 467-550 for
    the conversion): tdm_net_create decodes them to the half-rounded floats,
    and the FP32 net equals the oracle forward on those rounded weights."""
    path = str(tmp_path / "half.marvin")
    oracle.write_marvin(path, weights, dtype=np.float16)
    assert open(path, "rb").read(1) == b"\x00"  # type id 0: half
    rounded = {k: v.astype(np.float16).astype(np.float32) for k, v in weights.items()}
    net = tdm.Net(precision="fp32", marvin_path=path)
    got = net.forward(patches).cpu().numpy()
    p = patches.cpu().numpy()
    want = oracle.net_forward(p, rounded)
    assert rel_l2(got, want) <= 1e-4
    # and not the unrounded weights' output (half rounding moves descriptors ~1e-3)
    assert rel_l2(got, oracle.net_forward(p, weights)) > 10 * rel_l2(got, want)
    net.close()
    tdm.device_status()
