"""Device-resident fragment store: registering two stored fragments equals
tdm_register_pair on their points (the reference's describe-once,
register-many flow: getKeyptsAndDesc.m then register2Fragments.m); repeated
descriptions are hits that launch nothing; least recently used entries are
evicted when the budget is full."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KW = dict(max_points=160_000, max_keypoints=1000, max_voxels=120_000_000, match_precision="bf16",
          ransac_seed=5, ransac_iters=30_000)


@pytest.fixture(scope="module")
def net(tdm, oracle):
    return tdm.Net(oracle.he_normal_weights(20263000), precision="bf16")


def _key(r):
    return (tuple(r.rt), r.n_matches, r.n_inliers, r.best_trial, tuple(r.keypoints), tuple(map(tuple, r.grid_dim)))


def test_register_stored_equals_register_pair(tdm, net, scene, cuda):
    import torch
    a, b, _ = scene.fragment_pair(20263001, n_points=150_000)
    k, seed = 1000, 41
    pipe = tdm.Pipeline(net, **KW)
    want = _key(pipe.register(a, b, seed=seed, k=k))
    store = tdm.Store(256 << 20)
    assert not store.describe(pipe, 1, torch.from_numpy(a).to(cuda), seed, k)
    assert not store.describe(pipe, 2, torch.from_numpy(b).to(cuda), seed + 1, k)
    before = tdm.launch_count()
    assert store.describe(pipe, 1, torch.from_numpy(a).to(cuda), seed, k)  # hit: nothing runs
    assert tdm.launch_count() == before
    assert _key(tdm.register_stored(pipe, store, 1, 2)) == want
    # the stored descriptors are the fragment's descriptors
    kp, desc, g = store.get(1)
    kp2, desc2, g2 = pipe.describe(torch.from_numpy(a).to(cuda), seed, k)
    assert torch.equal(kp, kp2) and torch.equal(desc, desc2) and tuple(g.dim) == tuple(g2.dim)
    st = store.stats()
    assert st["entries"] == 2 and st["hits"] == 1 and st["misses"] == 2
    with pytest.raises(tdm.TdmError, match="no fragment"):
        tdm.register_stored(pipe, store, 1, 99)
    store.close()
    pipe.close()
    tdm.device_status()


def test_least_recently_used_entries_are_evicted(tdm, net, scene, cuda):
    import torch
    k = 200
    per = 256 * ((k * 12 + 255) // 256) + 256 * ((k * 2048 + 255) // 256)
    store = tdm.Store(3 * per)  # three entries
    pipe = tdm.Pipeline(net, **KW)
    pts = [torch.from_numpy(scene.fragment(20263100 + i, n_points=30_000)).to(cuda) for i in range(4)]
    for i in range(3):
        store.describe(pipe, 10 + i, pts[i], 1, k)
    store.describe(pipe, 10, pts[0], 1, k)  # touch entry 10: entry 11 is now the oldest
    store.describe(pipe, 13, pts[3], 1, k)
    st = store.stats()
    assert st["entries"] == 3 and st["evictions"] == 1
    with pytest.raises(tdm.TdmError):
        store.get(11)
    for key in (10, 12, 13):
        store.get(key)
    # a different keypoint count replaces the entry (a miss)
    assert not store.describe(pipe, 10, pts[0], 1, k - 10)
    assert store.get(10)[0].shape[0] == k - 10
    store.close()
    pipe.close()
    tdm.device_status()
