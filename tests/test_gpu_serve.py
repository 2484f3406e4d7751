"""Multi-stream serving of batched operators (umi_gb300/serve.py), with
requests in flight on several instances and collected in any order: every
request's outputs match the FP64 CPU oracle (same tolerances as the direct
operators, rel <= 1e-5) and equal the direct call of the same operator on its
images bit for bit (the served path adds no arithmetic of its own)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _bil_rel(got, want):
    return np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-3))


def _wf_rel(got, want, x, wts):
    h, w = x.shape
    p = np.pad(np.abs(x.astype(np.float64)), 1)
    s = np.zeros((h, w))
    for dy in range(3):
        for dx in range(3):
            s += np.abs(wts[:, :, dy, dx]) * p[dy:dy + h, dx:dx + w]
    return np.max(np.abs(got - want) / np.maximum(np.abs(want), s))


def _cv_rel(got, want, L, R, nd):
    c, h, w = L.shape
    Rp = np.concatenate([np.abs(R.astype(np.float64)), np.zeros((c, h, nd))], axis=2)
    La = np.abs(L.astype(np.float64))
    s = np.stack([(La * Rp[:, :, d:d + w]).sum(0) for d in range(nd)], axis=-1)
    return np.max(np.abs(got - want) / np.maximum(np.maximum(np.abs(want), s), 1e-30))


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("instances", [1, 3])
def test_bilateral_requests_match_oracle(umi, orc, dev, instances):
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
            assert _bil_rel(o, orc.bilateral_f64(x, 2, 2.0, 0.1)) <= TOL, i
            assert np.array_equal(o, umi.bilateral_f32(_t(x, dev), 2, 2.0, 0.1).cpu().numpy()), i
    with pytest.raises(KeyError):
        srv.result(tickets[0])
    # zero-copy results, consumed before the instance is reused
    t = srv.submit(reqs[0])
    view = srv.result(t, copy=False)
    assert np.array_equal(view[0], umi.bilateral_f32(_t(reqs[0][0], dev), 2, 2.0, 0.1).cpu().numpy())
    srv.close()


def test_wfilter_and_cost_volume_requests_match_oracle(umi, orc, dev):
    from umi_gb300 import serve
    g = np.random.default_rng(5)
    s = (40, 70)
    srv = serve.BatchServer(umi.OP_WFILTER_PP, [(s, s + (3, 3), s)], instances=2, device=dev)
    reqs = [(g.random(s, dtype=np.float32), g.random(s + (3, 3), dtype=np.float32)) for _ in range(4)]
    ts = [srv.submit([x], [w]) for x, w in reqs]
    for t, (x, w) in zip(ts, reqs):
        got = srv.result(t)[0]
        assert _wf_rel(got, orc.wfilter_pp_f64(x, w), x, w) <= TOL
        assert np.array_equal(got, umi.wfilter3x3_pp_f32(_t(x, dev), _t(w, dev)).cpu().numpy())
    srv.close()
    c, h, w = 32, 9, 150
    srv = serve.BatchServer(umi.OP_COST_VOLUME, [((c, h, w), (c, h, w), (h, w, 64))],
                            umi.BatchParams(0, 0.0, 0.0, c, 64), instances=2, device=dev)
    reqs = [(g.standard_normal((c, h, w)).astype(np.float32), g.standard_normal((c, h, w)).astype(np.float32))
            for _ in range(3)]
    ts = [srv.submit([L], [R]) for L, R in reqs]
    for t, (L, R) in zip(ts, reqs):
        got = srv.result(t)[0]
        assert _cv_rel(got, orc.cost_volume_dot_f64(L, R, 64), L, R, 64) <= TOL
        assert np.array_equal(got, umi.cost_volume_dot_f32(_t(L, dev), _t(R, dev), 64).cpu().numpy())
    with pytest.raises(ValueError):
        srv.submit([reqs[0][0]])  # the cost volume needs its right feature map
    srv.close()
