"""Batched form: many fragments of uneven point and keypoint counts and voxel
sizes through one persistent launch per stage (and a captured CUDA graph)
give, fragment by fragment, the bits of the single-fragment path.  The tile
autotuner changes no descriptor bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def weights(oracle):
    return oracle.he_normal_weights(20263000)


@pytest.fixture(scope="module")
def frags(scene):
    """Six fragments: 20k..90k points, 1 or 2 cm voxels, 40..260 keypoints."""
    rng = np.random.default_rng(77)
    out = []
    for f in range(6):
        n = int(np.exp(rng.uniform(np.log(20_000), np.log(90_000))))
        pts = scene.fragment(20263100 + f, n_points=n)
        vs = 0.01 if rng.random() < 0.5 else 0.02
        out.append((pts, vs, int(rng.integers(40, 260)), 1000 + 17 * f))
    out[1] = (out[1][0], 0.02, out[1][2], out[1][3])  # both voxel sizes present
    out[2] = (out[2][0], 0.01, out[2][2], out[2][3])
    return out


def _batch_inputs(frags, cuda):
    import torch
    pts = np.concatenate([p for p, _, _, _ in frags]).astype(np.float32)
    off = np.concatenate([[0], np.cumsum([p.shape[0] for p, _, _, _ in frags])])
    return (torch.from_numpy(pts).to(cuda), off, [v for _, v, _, _ in frags], [k for _, _, k, _ in frags],
            [s for _, _, _, s in frags])


def _single(tdm, net, frags, cuda):
    import torch
    out = []
    for pts, vs, k, seed in frags:
        pipe = tdm.Pipeline(net, voxel_size=vs, max_points=100_000, max_keypoints=300, max_voxels=80_000_000)
        kp, desc, g = pipe.describe(torch.from_numpy(pts).to(cuda), seed, k)
        out.append((kp.cpu().numpy(), desc.cpu().numpy(), g.as_tuple()))
        pipe.close()
    return out


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_batch_equals_single_fragments(tdm, weights, frags, cuda, precision):
    net = tdm.Net(weights, precision=precision)
    want = _single(tdm, net, frags, cuda)
    batch = tdm.Batch(net, max_fragments=8, max_points=600_000, max_keypoints=2_000, max_voxels=300_000_000,
                      use_graph=False)
    kp, desc, grids = batch.describe(*_batch_inputs(frags, cuda))
    kp, desc = kp.cpu().numpy(), desc.cpu().numpy()
    k0 = 0
    for f, (wkp, wdesc, wg) in enumerate(want):
        k = wkp.shape[0]
        assert grids[f].as_tuple() == wg, f
        assert np.array_equal(kp[k0:k0 + k], wkp), f
        assert np.array_equal(desc[k0:k0 + k], wdesc), f
        k0 += k
    batch.close()
    tdm.device_status()


def test_graph_replay_with_new_fragments(tdm, weights, frags, cuda, scene):
    """A captured graph replays for other points, voxel sizes and seeds with
    the same fragment count and total keypoints, and equals a direct run."""
    import torch
    net = tdm.Net(weights, precision="bf16")
    pts, off, vs, ks, seeds = _batch_inputs(frags, cuda)
    K = sum(ks)
    kp_buf = torch.empty((K, 3), dtype=torch.float32, device=cuda)
    desc_buf = torch.empty((K, 512), dtype=torch.float32, device=cuda)
    kw = dict(max_fragments=8, max_points=600_000, max_keypoints=2_000, max_voxels=300_000_000)
    g = tdm.Batch(net, use_graph=True, **kw)
    g.describe(pts, off, vs, ks, seeds, kp_buf, desc_buf)  # direct run, then capture
    assert not g.stats()["replayed"]
    # second set: other seeds, voxel sizes swapped, keypoints moved between fragments
    seeds2 = [s + 5 for s in seeds]
    vs2 = [0.03 - v for v in vs]
    ks2 = list(ks)
    ks2[0] += 10
    ks2[3] -= 10
    kp2, desc2, grids2 = g.describe(pts, off, vs2, ks2, seeds2, kp_buf, desc_buf)
    st = g.stats()
    assert st["replayed"] and st["launches_per_call"] > 0
    d = tdm.Batch(net, use_graph=False, **kw)
    kp3, desc3, grids3 = d.describe(pts, off, vs2, ks2, seeds2)
    assert [x.as_tuple() for x in grids2] == [x.as_tuple() for x in grids3]
    assert torch.equal(kp2, kp3) and torch.equal(desc2, desc3)
    # a tile change makes the captured forward stale: the next call captures anew
    net.set_tile("conv3", 64, 2)
    kp4, desc4, _ = g.describe(pts, off, vs2, ks2, seeds2, kp_buf, desc_buf)
    assert not g.stats()["replayed"]
    assert torch.equal(desc4, desc3)
    g.close()
    d.close()


def test_batch_limits(tdm, weights, frags, cuda):
    net = tdm.Net(weights, precision="bf16")
    pts, off, vs, ks, seeds = _batch_inputs(frags, cuda)
    small = tdm.Batch(net, max_fragments=8, max_points=600_000, max_keypoints=2_000, max_voxels=1_000_000,
                      use_graph=False)
    with pytest.raises(tdm.TdmError, match="max_voxels"):
        small.describe(pts, off, vs, ks, seeds)
    few = tdm.Batch(net, max_fragments=8, max_points=1_000, max_keypoints=2_000, max_voxels=300_000_000)
    with pytest.raises(tdm.TdmError, match="max_points"):
        few.describe(pts, off, vs, ks, seeds)
    bad = np.array(off)
    bad[2] = bad[1]  # an empty fragment
    ok = tdm.Batch(net, max_fragments=8, max_points=600_000, max_keypoints=2_000, max_voxels=300_000_000)
    with pytest.raises(tdm.TdmError, match="points"):
        ok.describe(pts, bad, vs, ks, seeds)
    # still usable after refusals
    kp, desc, _ = ok.describe(pts, off, vs, ks, seeds)
    assert np.isfinite(desc.cpu().numpy()).all()
    tdm.device_status()


@pytest.fixture(scope="module")
def patches(tdm, frags, cuda):
    import torch
    pts, vs = frags[0][0], frags[0][1]
    g = tdm.grid_from_points_host(pts, voxel_size=vs)
    pd = torch.from_numpy(pts).to(cuda)
    _, kg = tdm.keypoints(pd, tdm.keypoint_indices(9, pts.shape[0], 300, device=cuda), g)
    return tdm.gather(tdm.tdf(pd, g), g, kg)


@pytest.mark.parametrize("precision", ["bf16", "fp8"])
def test_autotune_keeps_descriptor_bits(tdm, weights, patches, precision):
    net = tdm.Net(weights, precision=precision)
    if precision == "fp8":
        net.calibrate(patches)
    before = net.forward(patches).cpu().numpy()
    tiles = net.autotune(patches, reps=2)
    forms = net.forms()
    for layer, (nt, ms) in tiles.items():
        if layer == "conv2":  # dx-fused: on a CTA pair (N = 192), or 32 outputs per CTA (N = 96)
            assert forms[layer] in ("dxf", "dxf_pair") and nt == 32 and ms in (1, 2), layer
        elif forms[layer] in ("gather", "xrun", "gather_wt", "xrun_wt"):  # one accumulator buffer allowed
            assert layer in ("conv3", "conv4", "conv5", "conv6", "conv7"), layer
            assert (nt, ms) in ((256, 2), (256, 1), (128, 2)), layer
        else:
            assert forms[layer] == "grid", layer
            assert nt in (64, 128, 256) and ms in (1, 2, 4) and 2 * nt * ms <= 512, layer
    after = net.forward(patches).cpu().numpy()
    assert np.array_equal(before, after)
    tdm.device_status()


@pytest.mark.parametrize("layer,tiles", [("conv2", [(32, 2, "dxf"), (32, 1, "dxf"), (32, 2, "dxf_pair")]),
                                         ("conv3", [(64, 4), (64, 2), (128, 2), (128, 1), (128, 2, "gather"),
                                                    (128, 2, "xrun"), (128, 2, "gather_wt"), (128, 2, "xrun_wt")]),
                                         ("conv4", [(128, 2, "gather"), (128, 2, "grid"), (128, 2, "xrun"),
                                                    (128, 2, "xrun_wt"), (128, 2, "gather_wt")]),
                                         ("conv5", [(256, 1, "gather"), (128, 2, "gather"), (256, 1, "grid"),
                                                    (256, 2, "xrun"), (256, 1, "xrun"), (128, 2, "xrun")]),
                                         ("conv6", [(64, 2), (128, 1), (256, 1), (256, 2, "gather"), (256, 2, "xrun")]),
                                         ("conv7", [(256, 1, "grid"), (128, 2, "gather"), (256, 1, "gather"),
                                                    (256, 2, "xrun"), (128, 2, "xrun")]),
                                         ("conv8", [(64, 4), (128, 2), (256, 1)])])
def test_every_tile_same_bits(tdm, weights, patches, layer, tiles):
    """Every tile and kernel form of a layer gives the same descriptor bits
    (the gathered-row form skips the grid form's dropped rows, nothing else)."""
    net = tdm.Net(weights, precision="bf16")
    ref = net.forward(patches).cpu().numpy()
    for t in tiles:
        net.set_tile(layer, *t)
        if len(t) == 3:
            assert net.forms()[layer] == t[2]
        assert np.array_equal(net.forward(patches).cpu().numpy(), ref), (layer, t)
    with pytest.raises(tdm.TdmError):
        net.set_tile("conv2", 128, 1)  # conv2 has 64 outputs


def test_fp8_gather_and_grid_forms_same_bits(tdm, weights, patches):
    """E4M3 operands: the grid, gathered-row and x-run forms of conv3..conv7 agree bit for bit."""
    net = tdm.Net(weights, precision="fp8")
    net.calibrate(patches)
    for layer in ("conv3", "conv4", "conv5", "conv6", "conv7"):
        net.set_tile(layer, 128, 2, "grid")
    ref = net.forward(patches).cpu().numpy()
    for layer in ("conv3", "conv4", "conv5", "conv6", "conv7"):
        net.set_tile(layer, 128, 2, "gather")
    assert set(net.forms()[k] for k in ("conv3", "conv4", "conv5", "conv6", "conv7")) == {"gather"}
    assert np.array_equal(net.forward(patches).cpu().numpy(), ref)
    for layer in ("conv5", "conv6", "conv7"):
        net.set_tile(layer, 256, 2, "gather")
    assert np.array_equal(net.forward(patches).cpu().numpy(), ref)
    for layer in ("conv3", "conv4", "conv5", "conv6", "conv7"):
        net.set_tile(layer, 128, 2, "xrun")
    assert np.array_equal(net.forward(patches).cpu().numpy(), ref)
    for form in ("xrun_wt", "gather_wt"):  # weights as the MMA's A operand, E4M3 output transposed
        for layer in ("conv3", "conv4"):
            net.set_tile(layer, 128, 2, form)
        assert np.array_equal(net.forward(patches).cpu().numpy(), ref), form
    tdm.device_status()


@pytest.mark.parametrize("precision", ["bf16", "fp8"])
def test_gathered_forms_small_batches(tdm, weights, patches, precision):
    """Tiny and ragged batches (one tile, partial tiles, x-run padding rows past
    the end) give every patch the bits it gets in a full batch, in every form."""
    net = tdm.Net(weights, precision=precision)
    if precision == "fp8":
        net.calibrate(patches)
    full = net.forward(patches).cpu().numpy()
    forms = [("gather", (128, 2), (256, 2)), ("xrun", (128, 2), (256, 2)), ("xrun_wt", (128, 2), None),
             ("gather_wt", (128, 2), None)]
    for form, t128, t256 in forms:
        for layer in ("conv3", "conv4", "conv5", "conv6", "conv7"):
            t = t128 if layer in ("conv3", "conv4") else t256
            if t is None:
                continue
            net.set_tile(layer, t[0], t[1], form)
        for lo, hi in ((7, 8), (0, 3), (100, 137)):
            got = net.forward(patches[lo:hi].contiguous()).cpu().numpy()
            assert np.array_equal(got, full[lo:hi]), (form, lo, hi)
    tdm.device_status()


@pytest.mark.parametrize("precision", ["bf16", "fp8"])
def test_conv2_pair_form_same_bits(tdm, weights, patches, precision):
    """conv2 on a CTA pair (one M = 256, N = 192 MMA over two SMs) against the
    single-CTA dx-fused form: the same descriptor, conv2 (unfused epilogue)
    and pool1 (x-pair max in the epilogue) bits, on full, tiny and ragged
    batches (tiles that straddle patches, the pair's second half past the
    last row)."""
    net = tdm.Net(weights, precision=precision)
    if precision == "fp8":
        net.calibrate(patches)
    assert net.forms()["conv2"] == "dxf_pair"  # the default
    out = {}
    for form, ms in (("dxf_pair", 2), ("dxf", 2), ("dxf", 1)):
        net.set_tile("conv2", 32, ms, form)
        assert net.forms()["conv2"] == form
        for lo, hi in ((0, 300), (7, 8), (0, 3), (100, 137)):
            b = patches[lo:hi].contiguous()
            out[(form, ms, lo, hi, "desc")] = net.forward(b).cpu().numpy()
            if hi - lo <= 37:
                out[(form, ms, lo, hi, "conv2")] = net.response("conv2", b).cpu().numpy()
                out[(form, ms, lo, hi, "pool1")] = net.response("pool1", b).cpu().numpy()
    for key, v in out.items():
        if key[0] != "dxf_pair":
            ref = out[("dxf_pair", 2) + key[2:]]
            assert np.array_equal(v, ref), key
    tdm.device_status()
