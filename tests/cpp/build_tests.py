"""Build the C++/CUDA test programs of tests/cpp/ (sm_103a) into tests/cpp/_bin/.

Called by __graft_entry__.build(); each program links libumi_gb300.so.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
BIN = os.path.join(HERE, "_bin")
PROGRAMS = ["dropin_apps", "generic_fuzz", "checked_oob"]
EXTRA_FLAGS = {"checked_oob": ["-DUMI_CHECKED"]}

sys.path.insert(0, ROOT)


def binary(name: str) -> str:
    return os.path.join(BIN, name)


def _build_one(name: str) -> str:
    from umi_gb300 import build as B
    src = os.path.join(HERE, name + ".cu")
    out = binary(name)
    deps = [src, B.LIB] + [os.path.join(ROOT, "include", "umi", f) for f in ("UMI.h", "UMI_gpu.h")] + [
        os.path.join(ROOT, "include", "umi_gb300.h"), os.path.join(ROOT, "oracle", "umi_interp.hpp")]
    if os.path.exists(out) and all(os.path.getmtime(d) <= os.path.getmtime(out) for d in deps if os.path.exists(d)):
        return out
    cmd = [B.nvcc()] + B.ARCH + EXTRA_FLAGS.get(name, []) + ["-std=c++17", "-O2", "-lineinfo", "-I",
                                                            os.path.join(ROOT, "include"), src, "-o", out,
                                 "-L", os.path.dirname(B.LIB), "-lumi_gb300", "-Xlinker",
                                 "-rpath," + os.path.dirname(B.LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr[-4000:]}")
    return out


def build() -> list[str]:
    os.makedirs(BIN, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(PROGRAMS)) as ex:
        return list(ex.map(_build_one, PROGRAMS))


if __name__ == "__main__":
    print(build())
