"""Host-side logic of bench.py without a GPU: the max-over-ranks reduction
on world_size 2 (gloo, CPU) and the reference arm's JSON line."""
import json
import os
import subprocess
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    v = bench.max_over_ranks(1.5 + rank, world, torch.device("cpu"))
    bench.barrier(world)
    out[rank] = v
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    port = 29500 + (os.getpid() % 1000)
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert dict(out) == {0: 2.5, 1: 2.5}


def test_reference_arm_prints_one_json_line(built):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "sand_column_32k", "--steps", "2", "--warmup", "1"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0


def test_profiled_traffic_is_consistent():
    """The per-substep DRAM traffic that bench.py reports as roofline.traffic
    (an ncu capture of one substep) is the sum of its kernels' reads and
    writes, and above the algorithmic bytes it is compared with."""
    sys.path.insert(0, ROOT)
    import bench

    t = bench.profiled_traffic("sand_column_1m")
    assert t is not None
    total = sum(k["dram_read_MB"] + k["dram_write_MB"] for k in t["kernels"].values()) * 1e6
    assert abs(total - t["bytes_per_substep"]) < 1e-3 * t["bytes_per_substep"]
    assert t["algorithmic_bytes_per_substep"] == 284 * 1048576
    assert t["bytes_per_substep"] > t["algorithmic_bytes_per_substep"]
