"""CPU checks of the learned motion proposal: the FP64 oracle's gradient
against central finite differences, and checkpoint save / load / resume."""
import numpy as np
import pytest

from oracle import menet


def _case(seed=0, h=32, w=48):
    import umi_gb300
    g = np.random.default_rng(seed)
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = g.integers(0, 256, (h, w), dtype=np.uint8)
    p = umi_gb300.init_params(seed + 1)
    layers, wh, bh, _ = menet.layout()
    p[wh:bh] = g.normal(0, 0.2, bh - wh)
    for _, bo in layers:
        p[bo:bo + menet.CH] = g.normal(0, 0.05, menet.CH)
    tgt = g.integers(-40, 40, ((h // 16) * (w // 16), 2)).astype(np.int32)
    return cur, ref, p.astype(np.float32), tgt


def test_layout_matches_library_layout():
    import umi_gb300
    assert umi_gb300.param_layout() == menet.layout()


def test_oracle_gradient_matches_finite_differences():
    cur, ref, p, tgt = _case()
    _, grad = menet.loss_and_grad(p, cur, ref, tgt, bf16=False)
    layers, wh, bh, total = menet.layout()
    q = p.astype(np.float64)

    def loss(x):
        ws = [x[wo:bo].reshape(menet.CH, c, 9) for (wo, bo), c in zip(layers, menet.CIN)]
        a = menet.downsample(cur, ref)
        for l in range(4):
            a = np.maximum(menet.conv(a, ws[l], x[layers[l][1]:layers[l][1] + menet.CH], menet.DIL[l]), 0.0)
        pred = menet.head_features(a, cur.shape[0] // 16, cur.shape[1] // 16) @ x[wh:bh].reshape(2, -1).T + x[bh:bh + 2]
        e = np.abs(pred - tgt / 16.0)
        return np.where(e < 1, 0.5 * e * e, e - 0.5).sum() / pred.shape[0]

    g = np.random.default_rng(5)
    idx = [layers[0][0], layers[0][1], layers[1][0] + 7, layers[3][1] + 3, wh + 11, bh, bh + 1]
    idx += [int(i) for i in g.choice(total, 24, replace=False)]
    eps = 1e-6
    for i in idx:
        hi = q.copy(); hi[i] += eps
        lo = q.copy(); lo[i] -= eps
        fd = (loss(hi) - loss(lo)) / (2 * eps)
        assert abs(fd - grad[i]) <= 1e-7 + 1e-5 * abs(fd), (i, fd, grad[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 65504.0], np.float32)
    r = menet.to_bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12


def test_checkpoint_roundtrip_and_resume(tmp_path):
    from umi_gb300 import menet_train as T
    cur, ref, p, tgt = _case(3)
    m = np.zeros_like(p); v = np.zeros_like(p)
    straight = (p.copy(), m.copy(), v.copy())
    for step in range(1, 4):
        _, g = menet.loss_and_grad(straight[0], cur, ref, tgt)
        straight = menet.adam_step(*straight[:1], g, *straight[1:], step=step, lr=1e-3)
    q, mm, vv = p.copy(), m.copy(), v.copy()
    for step in range(1, 3):
        _, g = menet.loss_and_grad(q, cur, ref, tgt)
        q, mm, vv = menet.adam_step(q, g, mm, vv, step=step, lr=1e-3)
    path = str(tmp_path / "ck.bin")
    T.save_checkpoint(path, q, mm, vv, step=2)
    ck = T.load_checkpoint(path)
    assert ck["step"] == 2
    assert np.array_equal(ck["params"], q) and np.array_equal(ck["m"], mm) and np.array_equal(ck["v"], vv)
    _, g = menet.loss_and_grad(ck["params"], cur, ref, tgt)
    resumed = menet.adam_step(ck["params"], g, ck["m"], ck["v"], step=ck["step"] + 1, lr=1e-3)
    for a, b in zip(resumed, straight):
        assert np.array_equal(a, b)


def test_checkpoint_rejects_bad_files(tmp_path):
    from umi_gb300 import menet_train as T
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"NOTMENET" + bytes(16))
    with pytest.raises(ValueError):
        T.load_checkpoint(str(bad))
    good = tmp_path / "good.bin"
    T.save_checkpoint(str(good), np.ones(10, np.float32))
    good.write_bytes(good.read_bytes()[:-4])
    with pytest.raises(ValueError, match="truncated"):
        T.load_checkpoint(str(good))


def test_committed_weights_load():
    import os
    from umi_gb300 import menet_train as T
    import umi_gb300
    if not os.path.exists(T.WEIGHTS):
        pytest.skip("no trained weights committed")
    ck = T.load_checkpoint(T.WEIGHTS)
    assert ck["params"].size == menet.layout()[3] and np.isfinite(ck["params"]).all()
