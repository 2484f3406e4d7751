"""Multi-stream serving of batched operators (umi_gb300/serve.py): every
request's outputs equal the direct call of the same operator on its images,
with requests in flight on several instances, collected in any order."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("instances", [1, 3])
def test_bilateral_requests_match_direct_calls(umi, dev, instances):
    from umi_gb300 import serve
    shapes = [(64, 80), (33, 129), (1, 1)]
    prm = umi.BatchParams(2, 2.0, 0.1, 0, 0)
    srv = serve.BatchServer(umi.OP_BILATERAL, [(s, None, s) for s in shapes], prm, instances=instances, device=dev)
    g = np.random.default_rng(instances)
    reqs = [[g.random(s, dtype=np.float32) for s in shapes] for _ in range(7)]
    tickets = [srv.submit(r) for r in reqs]
    order = list(range(7))
    g.shuffle(order)
    for i in order:
        out = srv.result(tickets[i])
        for x, o in zip(reqs[i], out):
            want = umi.bilateral_f32(_t(x, dev), 2, 2.0, 0.1).cpu().numpy()
            assert np.array_equal(o, want), i
    with pytest.raises(KeyError):
        srv.result(tickets[0])
    # zero-copy results, consumed before the instance is reused
    t = srv.submit(reqs[0])
    view = srv.result(t, copy=False)
    assert np.array_equal(view[0], umi.bilateral_f32(_t(reqs[0][0], dev), 2, 2.0, 0.1).cpu().numpy())
    srv.close()


def test_wfilter_and_cost_volume_requests(umi, dev):
    from umi_gb300 import serve
    g = np.random.default_rng(5)
    s = (40, 70)
    srv = serve.BatchServer(umi.OP_WFILTER_PP, [(s, s + (3, 3), s)], instances=2, device=dev)
    reqs = [(g.random(s, dtype=np.float32), g.random(s + (3, 3), dtype=np.float32)) for _ in range(4)]
    ts = [srv.submit([x], [w]) for x, w in reqs]
    for t, (x, w) in zip(ts, reqs):
        assert np.array_equal(srv.result(t)[0], umi.wfilter3x3_pp_f32(_t(x, dev), _t(w, dev)).cpu().numpy())
    srv.close()
    c, h, w = 32, 9, 150
    srv = serve.BatchServer(umi.OP_COST_VOLUME, [((c, h, w), (c, h, w), (h, w, 64))],
                            umi.BatchParams(0, 0.0, 0.0, c, 64), instances=2, device=dev)
    reqs = [(g.standard_normal((c, h, w)).astype(np.float32), g.standard_normal((c, h, w)).astype(np.float32))
            for _ in range(3)]
    ts = [srv.submit([L], [R]) for L, R in reqs]
    for t, (L, R) in zip(ts, reqs):
        assert np.array_equal(srv.result(t)[0], umi.cost_volume_dot_f32(_t(L, dev), _t(R, dev), 64).cpu().numpy())
    with pytest.raises(ValueError):
        srv.submit([reqs[0][0]])  # the cost volume needs its right feature map
    srv.close()
