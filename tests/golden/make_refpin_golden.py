"""Generate tests/golden/refpin.json from the reference's own example programs.

Run in a checkout where the reference sources are available (the directory
named by UMI_REFERENCE, else `reference` beside this repository):

    python tests/golden/make_refpin_golden.py

Steps:
 1. `make -C oracle refpin` compiles every main/<app>.cu of the reference, as
    plain C++, against the oracle shim (oracle/refpin/): each UMI::Execute call
    runs on the CPU oracle interpreter.
 2. Every program runs with UMI_REFPIN_DUMP set; it exits 0 only if its own
    CPU check (the assert loop at the end of main/<app>.cu) accepted the
    oracle's result.  The raw outputs of every Execute call are dumped.
 3. The closed-form oracle (liboracle.so) recomputes each output from the
    same inputs and must match the dump bit for bit.
 4. The SHA-256, element count, sum and first values of each output are
    written to refpin.json, which the GPU drop-in tests compare against.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

REF = os.environ.get("UMI_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))

# Parameters and inputs of each example program (main/<app>.cu).
APPS = {
    "filter3x3": dict(h=300, w=500, init=-5, mul=2, pad=999, input="iota", dtype="int32"),
    "wfilter3x3": dict(h=250, w=300, init=-5, pad=56, weights=[1, 2, 1, 2, 4, 2, 1, 2, 1], input="iota", dtype="int32"),
    "bilateral": dict(h=250, w=300, sigma_s=4.0, sigma_r=10.0, ofs=12, input="iota", dtype="float32"),
    "cost_volume": dict(h=1080, w=1920, k=7, sr=15, input="iota", dtype="int32"),
    "full_me": dict(h=1080, w=1920, b=8, sr_ofs=-7, sr=15, input="iota", dtype="int32"),
    "iimg": dict(h=300, w=500, input="ones", dtype="int32"),
    "gemm": dict(m=100, k=100, n=200, input="iota", dtype="int32"),
    "fprop": dict(n=32, c=40, ih=64, iw=80, k=60, f=7, s=2, ofs=-3, input="minstd_uniform_0_10", dtype="int32"),
}


def closed_form(app: str, p: dict) -> list[np.ndarray]:
    """Outputs of every Execute call of `app`, from the closed-form oracle."""
    if app == "filter3x3":
        x = np.arange(p["h"] * p["w"], dtype=np.int32).reshape(p["h"], p["w"])
        return [oracle.ref_filter3x3_i32(x, p["init"], p["mul"], p["pad"])]
    if app == "wfilter3x3":
        x = np.arange(p["h"] * p["w"], dtype=np.int32).reshape(p["h"], p["w"])
        return [oracle.ref_wfilter3x3_i32(x, p["weights"], p["init"], p["pad"])]
    if app == "bilateral":
        x = np.arange(p["h"] * p["w"], dtype=np.float32).reshape(p["h"], p["w"])
        ofs = p["ofs"]
        n1 = np.float32(-1.0) / (np.float32(2.0) * np.float32(p["sigma_s"]) ** 2)
        n2 = np.float32(-1.0) / (np.float32(2.0) * np.float32(p["sigma_r"]) ** 2)
        # main/bilateral.cu:45-48: w[i] = exp(d*d*norm_1) in double, stored as float
        ws = np.array([np.exp(float((i - ofs) * (i - ofs)) * float(n1)) for i in range(2 * ofs + 1)], np.float32)
        return [oracle.ref_bilateral_f32(x, ofs, ws, float(n2))]
    if app == "cost_volume":
        x = np.arange(p["h"] * p["w"], dtype=np.int32).reshape(p["h"], p["w"])
        return [oracle.ref_cost_volume_i32(x, p["k"], p["sr"])]
    if app == "full_me":
        x = np.arange(p["h"] * p["w"], dtype=np.int32).reshape(p["h"], p["w"])
        return [oracle.ref_full_me_i32(x, x, p["b"], p["sr_ofs"], p["sr"])]
    if app == "iimg":
        x = np.ones((p["h"], p["w"]), np.int32)
        rows = np.cumsum(x, axis=1, dtype=np.int32)
        return [np.ascontiguousarray(rows.T), oracle.ref_iimg_i32(x)]
    if app == "gemm":
        A = np.arange(p["m"] * p["k"], dtype=np.int32).reshape(p["m"], p["k"])
        B = np.arange(p["k"] * p["n"], dtype=np.int32).reshape(p["k"], p["n"])
        return [oracle.ref_gemm_i32(A, B)]
    if app == "fprop":
        n_in = p["n"] * p["c"] * p["ih"] * p["iw"]
        n_wt = p["k"] * p["c"] * p["f"] * p["f"]
        a, b = oracle.ref_fprop_inputs(n_in, n_wt)
        x = a.reshape(p["n"], p["c"], p["ih"], p["iw"])
        wt = b.reshape(p["k"], p["c"], p["f"], p["f"])
        return [oracle.ref_fprop_i32(x, wt, p["f"], p["s"], p["ofs"])]
    raise KeyError(app)


def digest(a: np.ndarray) -> dict:
    a = np.ascontiguousarray(a)
    return {
        "sha256": hashlib.sha256(a.tobytes()).hexdigest(),
        "n": int(a.size),
        "dtype": str(a.dtype),
        "sum": float(a.astype(np.float64).sum()),
        "head": [float(v) for v in a.ravel()[:8]],
    }


def main() -> None:
    if not os.path.isdir(os.path.join(REF, "main")):
        sys.exit(f"reference sources not found at {REF}")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}", "refpin"], check=True)
    out = {"generator": "tests/golden/make_refpin_golden.py", "apps": {}}
    with tempfile.TemporaryDirectory() as tmp:
        for app, p in APPS.items():
            env = dict(os.environ, UMI_REFPIN_DUMP=tmp, UMI_REFPIN_APP=app)
            r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", app)], env=env,
                               capture_output=True, text=True, timeout=3600)
            if r.returncode != 0:
                sys.exit(f"{app}: reference check failed (rc={r.returncode}) {r.stderr[-400:]}")
            outs = closed_form(app, p)
            calls = []
            for ci, want in enumerate(outs):
                raw = np.fromfile(os.path.join(tmp, f"{app}.{ci}.out0.bin"), dtype=want.dtype)
                if raw.size != want.size or not np.array_equal(raw, want.ravel()):
                    sys.exit(f"{app} call {ci}: closed-form oracle disagrees with the pinned interpreter")
                calls.append(digest(want))
            out["apps"][app] = {"params": p, "calls": calls}
            print(f"{app}: reference check passed, closed form matches ({len(calls)} call(s))")
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "refpin.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
