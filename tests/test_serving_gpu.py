"""Serving loop: requests of different sizes run concurrently on several slots;
each result equals the same request run alone (bit for bit: every kernel is
deterministic and every slot owns its buffers)."""
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
    return (tuple(r.rt), r.n_matches, r.n_inliers, r.best_trial)


def test_results_equal_alone_and_in_the_mix(tdm, net, requests):
    pipe = tdm.Pipeline(net, **KW)
    alone = [_key(pipe.register(a, b, seed=s, k=k)) for a, b, s, k in requests]
    pipe.close()
    srv = tdm.Server(net, slots=3, **KW)
    assert srv.slots == 3
    tickets = [srv.submit(a, b, s, k) for a, b, s, k in requests * 2]  # twelve requests, three at a time
    got = [srv.wait(t) for t in tickets]
    srv.close()
    for i, (r, lat) in enumerate(got):
        assert _key(r) == alone[i % len(requests)], i
        assert lat > 0
    tdm.device_status()


def test_admission_limits(tdm, net, requests):
    with pytest.raises(tdm.TdmError, match="budget"):
        tdm.Server(net, slots=2, hbm_budget_bytes=1 << 20, **KW)
    srv = tdm.Server(net, slots=64, hbm_budget_bytes=3 * (16 << 30), **KW)
    assert 1 <= srv.slots < 64  # the budget, not the request, bounds the slot count
    a, b, s, k = requests[0]
    with pytest.raises(tdm.TdmError, match="slot limits"):
        srv.submit(a, b, s, 5000)
    srv.close()
