"""The autotuner's cache (umi_gb300/autotune.py) on CPU, with the native sweep
faked: the first call per (GPU, op, size class) measures, later calls read
the cache, and a cached winner is measured again when the operator's number
of variants changes."""
import pytest


class _T:
    def __init__(self, h, w):
        self.shape = (h, w)


def test_cache_hits_and_invalidation(tmp_path, monkeypatch):
    torch = pytest.importorskip("torch")
    import umi_gb300 as U
    from umi_gb300 import autotune
    monkeypatch.setenv("UMI_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(torch.cuda, "get_device_name", lambda *a: "fake GB300")
    calls = []
    nvar = {"n": 4}

    def fake_tune(op, images, params=None, reps=3, stream=None):
        calls.append(op)
        return len(calls) % nvar["n"], 1.5

    monkeypatch.setattr(U, "autotune_batch", fake_tune)
    monkeypatch.setattr(U, "batch_variants", lambda op: nvar["n"])
    imgs = [(_T(256, 512), None, None)] * 3
    v1, ms, cached = autotune.tuned_variant(U.OP_BILATERAL, imgs)
    assert not cached and len(calls) == 1
    v2, _, cached = autotune.tuned_variant(U.OP_BILATERAL, imgs)
    assert cached and v2 == v1 and len(calls) == 1
    # another size class measures again
    autotune.tuned_variant(U.OP_BILATERAL, [(_T(2048, 2048), None, None)] * 3)
    assert len(calls) == 2
    # the operator gains a variant: the cached winner is re-measured
    nvar["n"] = 5
    _, _, cached = autotune.tuned_variant(U.OP_BILATERAL, imgs)
    assert not cached and len(calls) == 3
    assert autotune.size_class([]) == "empty"
