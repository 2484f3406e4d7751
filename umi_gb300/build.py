"""Build libumi_gb300.so (sm_103a) in place with nvcc.

    python -m umi_gb300.build          # or umi_gb300.build.build()

Every translation unit under umi_gb300/csrc/ is compiled in parallel into
umi_gb300/_build/, then linked into umi_gb300/libumi_gb300.so.  Objects are
rebuilt only when a source or header is newer.  One -gencode: sm_103a.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libumi_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def common_flags() -> list[str]:
    return ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
            + glob.glob(os.path.join(INCLUDE, "*.h")) + glob.glob(os.path.join(INCLUDE, "umi", "*.h")))


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not _newer(obj, [src] + _headers()):
        return obj
    cmd = [nvcc()] + ARCH + common_flags() + ["-c", src, "-o", obj]
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"] if verbose else []
    else:
        cmd += ["-x", "c++"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile and link libumi_gb300.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    _link(LIB, objs)
    return LIB


PROBE_DIR = os.path.join(ROOT, "probe")
PROBE_LIB = os.path.join(PROBE_DIR, "libumi_probe.so")


def _link(lib: str, objs: list[str]) -> None:
    if _newer(lib, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", lib] + objs + [
            "-Xlinker", "-rpath," + os.path.join(cuda_home(), "lib64")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")


def build_probe(verbose: bool = False) -> str:
    """The benchmark's instruction-throughput probes (probe/ beside bench.py),
    a library of their own, separate from the operator ABI."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(PROBE_DIR, "*.cu")))
    objs = [_compile(s, verbose) for s in srcs]
    _link(PROBE_LIB, objs)
    return PROBE_LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
