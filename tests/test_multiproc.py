"""Multi-process paths of bench.py on CPU (gloo, world size 2).

The operator has no exchange step, so N GPUs run N independent replicas; what
needs testing is the host side: rank 0 alone prints one JSON line, the others
exit 0, and the timing is the maximum over ranks."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_under_torchrun_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--workload", "filter3x3_1024", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["gpu_launches"] == 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


def _max_worker(rank, world, port, values, out_path):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist("gloo")
    d.barrier()
    m = d.max(values[rank])
    d.done()
    with open(f"{out_path}.{rank}", "w") as f:
        f.write(repr(m))


def test_dist_max_over_ranks(tmp_path):
    import torch.multiprocessing as mp
    values = [3.25, 7.5]
    port = _free_port()
    out = str(tmp_path / "max")
    mp.spawn(_max_worker, args=(2, port, values, out), nprocs=2, join=True)
    for rank in range(2):
        assert float(open(f"{out}.{rank}").read()) == max(values)


def test_single_process_dist_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        d = bench.Dist("gloo")
        assert d.world == 1 and d.rank == 0 and d.max(2.5) == 2.5
        d.barrier()
        d.done()
    finally:
        os.environ.update(env)


WORKLOADS = ["int_pair_1080p", "filter3x3_1024", "batched_uneven", "gemm_4096", "fprop_n32", "learned_me_4k",
             "coarse_me_4k", "video_y4m_1080p", "apps_1080p", "serve_bilateral_8x512"]


@pytest.mark.parametrize("workload", WORKLOADS)
def test_reference_arm_line_per_workload(workload):
    """Every workload's reference arm (the reference's CPU path, restated in
    the oracle) prints one line with the keys of the bench contract, on the
    same metric and config as the GPU arm."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", workload,
           "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline", "gpu_launches"):
        assert key in d, key
    assert d["impl"] == "reference" and d["config"]["workload"] == workload and d["value"] > 0
    assert d["e2e"]["value"] == d["value"] and d["cpu_baseline"]["kind"] in ("port", "reference")
