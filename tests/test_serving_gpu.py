"""Serving loop (continuous batching): requests of different sizes are taken
in waves by their own device footprint, the fragments of a wave are
described together by the batched kernels, and a second thread registers the
pairs from the device-resident store while the next wave is described.  Each
result equals the same request run alone (bit for bit); keyed fragments are
described once; queued requests can be cancelled; waits take a timeout."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KW = dict(max_points=70_000, max_keypoints=600, max_voxels=80_000_000, match_precision="bf16",
          ransac_seed=11, ransac_iters=20_000)


@pytest.fixture(scope="module")
def requests(scene):
    rng = np.random.default_rng(4)
    out = []
    for i in range(6):
        n = int(rng.integers(20_000, 70_000))
        a, b, _ = scene.fragment_pair(20261000 + i, n_points=n)
        out.append((a, b, 100 + i, int(rng.integers(200, 600))))
    return out


@pytest.fixture(scope="module")
def net(tdm, oracle):
    return tdm.Net(oracle.he_normal_weights(20261000), precision="bf16")


def _key(r):
    return (tuple(r.rt), r.n_matches, r.n_inliers, r.best_trial, tuple(r.keypoints))


def test_results_equal_alone_and_in_the_mix(tdm, net, requests):
    pipe = tdm.Pipeline(net, **KW)
    alone = [_key(pipe.register(a, b, seed=s, k=k)) for a, b, s, k in requests]
    pipe.close()
    srv = tdm.Server(net, slots=4, **KW)
    assert srv.slots == 4
    tickets = [srv.submit(a, b, s, k) for a, b, s, k in requests * 2]  # twelve requests at once
    got = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    for i, (r, lat) in enumerate(got):
        assert _key(r) == alone[i % len(requests)], i
        assert lat > 0
    assert st["requests_done"] == 12 and st["fragments_described"] == 24
    assert st["max_wave_requests"] >= 2 and st["waves"] < 12  # requests shared description launches
    print("serving stats:", st)
    tdm.device_status()


def test_keyed_fragments_are_described_once(tdm, net, scene):
    """All six pairs of four keyed views: four descriptions, six
    registrations, each equal to registering the stored fragments directly."""
    views = [scene.fragment(20262000 + i, n_points=40_000) for i in range(4)]
    k = 300
    srv = tdm.Server(net, slots=8, **KW)
    pairs = [(i, j) for i in range(4) for j in range(i + 1, 4)]
    frag = lambda i: {"key": 1000 + i, "pts": views[i], "seed": 70 + i, "k": k}
    tickets = [srv.submit_pair(frag(i), frag(j)) for i, j in pairs]
    got = [_key(srv.wait(t)[0]) for t in tickets]
    # later requests may name the stored views without their points
    t = srv.submit_pair({"key": 1000, "pts": None, "seed": 70, "k": k}, {"key": 1003, "pts": None, "seed": 73, "k": k})
    again = _key(srv.wait(t)[0])
    st = srv.stats()
    srv.close()
    assert st["fragments_described"] == 4, st
    assert again == got[pairs.index((0, 3))]
    import torch
    pipe = tdm.Pipeline(net, **KW)
    store = tdm.Store(64 << 20)
    for i in range(4):
        store.describe(pipe, 1000 + i, torch.from_numpy(views[i]).cuda(), 70 + i, k)
    for (i, j), g in zip(pairs, got):
        assert _key(tdm.register_stored(pipe, store, 1000 + i, 1000 + j)) == g, (i, j)
    store.close()
    pipe.close()
    tdm.device_status()


def test_cancel_and_wait_timeout(tdm, net, requests):
    srv = tdm.Server(net, slots=1, **KW)
    tickets = [srv.submit(a, b, s, k) for a, b, s, k in requests[:4]]
    srv.cancel(tickets[-1])  # still queued behind the first three (one request per wave)
    with pytest.raises(tdm.TdmError) as e:
        srv.wait(tickets[-1])
    assert e.value.status == 7  # CANCELLED
    left = list(tickets[:3])
    try:
        srv.wait(tickets[2], timeout_ms=0)  # most likely not finished yet
        left.remove(tickets[2])
    except tdm.TdmError as e2:
        assert e2.status == 6  # TIMEOUT: the ticket stays valid
    for t in left:
        r, _ = srv.wait(t, timeout_ms=60_000)
        assert r.n_matches > 0
    with pytest.raises(tdm.TdmError, match="unknown ticket"):
        srv.wait(10_000)
    assert srv.stats()["requests_cancelled"] == 1
    srv.close()
    tdm.device_status()


def test_admission_limits(tdm, net, requests):
    with pytest.raises(tdm.TdmError, match="budget"):
        tdm.Server(net, slots=2, hbm_budget_bytes=1 << 20, **KW)
    srv = tdm.Server(net, slots=64, hbm_budget_bytes=24 << 30, **KW)
    assert 1 <= srv.slots < 64  # the budget, not the request count, bounds a wave
    a, b, s, k = requests[0]
    with pytest.raises(tdm.TdmError, match="keypoints"):
        srv.submit(a, b, s, 5000)
    srv.close()
