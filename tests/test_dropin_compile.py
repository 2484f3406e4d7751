"""The reference's example programs compile unchanged against this library's
headers for sm_103a (include/umi/UMI_gpu.h + SyncedMemory.h, linked with
libumi_gb300.so).  Runs where the reference sources are present (they are
only read, in place; binaries go to a temporary folder)."""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("UMI_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
APPS = ["filter3x3", "wfilter3x3", "bilateral", "cost_volume", "full_me", "iimg", "gemm", "fprop"]


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "main")), reason="reference sources not present")
def test_reference_programs_compile_against_gpu_headers(tmp_path, umi):
    from umi_gb300 import build as B

    def compile_one(app):
        cmd = [B.nvcc()] + B.ARCH + ["-std=c++17", "-I", os.path.join(ROOT, "include", "umi"), "-I",
                                     os.path.join(ROOT, "include"), os.path.join(REF, "main", app + ".cu"), "-o",
                                     str(tmp_path / app), "-L", os.path.dirname(B.LIB), "-lumi_gb300"]
        return app, subprocess.run(cmd, capture_output=True, text=True)

    with ThreadPoolExecutor(max_workers=8) as ex:
        for app, r in ex.map(compile_one, APPS):
            assert r.returncode == 0, f"{app}: {r.stderr[-2000:]}"
            assert os.path.exists(tmp_path / app)
