"""GPU tests of the generic path (UMI::Execute, include/umi/UMI_gpu.h).

* The eight example applications of the reference, with the reference's
  descriptors and inputs (tests/cpp/dropin_apps.cu), run on the GPU; every
  integer output must have the SHA-256 digest that the reference's own CPU
  check accepted (tests/golden/refpin.json).  bilateral is float (expf on the
  device): it is held to the reference's own tolerance, 0.1 % relative
  (main/bilateral.cu:122), against the restated CPU loop.
* Randomised descriptors (tests/cpp/generic_fuzz.cu): GPU and CPU oracle
  interpreter must agree exactly and reject the same invalid descriptors.
"""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "refpin.json")))


def _bin(name):
    import sys
    sys.path.insert(0, os.path.join(HERE, "cpp"))
    import build_tests
    path = build_tests.binary(name)
    if not os.path.exists(path):
        build_tests.build()
    return path


@pytest.fixture(scope="module")
def dropin_run(tmp_path_factory, umi):
    out = tmp_path_factory.mktemp("dropin")
    r = subprocess.run([_bin("dropin_apps"), str(out)], capture_output=True, text=True, timeout=900)
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    return out, r, lines


@pytest.mark.parametrize("app", ["filter3x3", "wfilter3x3", "cost_volume", "full_me", "iimg", "gemm", "fprop"])
def test_dropin_app_matches_reference_check(dropin_run, app):
    out, r, lines = dropin_run
    assert r.returncode == 0, r.stderr + r.stdout
    calls = GOLD["apps"][app]["calls"]
    for ci, want in enumerate(calls):
        raw = np.fromfile(os.path.join(out, f"{app}.{ci}.bin"), dtype=np.int32)
        assert raw.size == want["n"], (app, ci)
        assert hashlib.sha256(raw.tobytes()).hexdigest() == want["sha256"], (app, ci)
    for l in lines:
        if l["app"] == app:
            assert l["status"] == 0 and l["cuda"] == "cudaSuccess"


def test_dropin_bilateral_within_reference_tolerance(dropin_run, orc):
    out, r, _ = dropin_run
    assert r.returncode == 0, r.stderr
    p = GOLD["apps"]["bilateral"]["params"]
    h, w, ofs = p["h"], p["w"], p["ofs"]
    got = np.fromfile(os.path.join(out, "bilateral.0.bin"), dtype=np.float32).reshape(h, w)
    x = np.arange(h * w, dtype=np.float32).reshape(h, w)
    n1 = np.float32(-1.0) / (np.float32(2.0) * np.float32(p["sigma_s"]) ** 2)
    n2 = np.float32(-1.0) / (np.float32(2.0) * np.float32(p["sigma_r"]) ** 2)
    ws = np.array([np.exp(float((i - ofs) ** 2) * float(n1)) for i in range(2 * ofs + 1)], np.float32)
    want = orc.ref_bilateral_f32(x, ofs, ws, float(n2))
    ratio = want / got
    assert np.all((ratio > 0.999) & (ratio < 1.001))


def test_generic_fuzz_against_oracle(umi):
    r = subprocess.run([_bin("generic_fuzz"), "700", "2024"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:] + r.stdout
    s = json.loads(r.stdout.strip().splitlines()[-1])
    assert s["failures"] == 0 and s["trials"] == 700 and s["rejected_as_expected"] >= 100
