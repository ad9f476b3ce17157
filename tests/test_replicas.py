"""The multi-rank bench path on CPU: bench.py --gpus N runs N independent replicas of
the single-GPU loop (the path does not shard), so what spans ranks is the timing
reduction (the slowest replica's time, on every rank) and the launch contract of the
reference arm (rank 0 runs and prints one JSON line, the other ranks exit 0 without
output)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, values, out):
    import importlib.util
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    spec = importlib.util.spec_from_file_location("bench_rank", os.path.join(ROOT, "bench.py"))
    b = importlib.util.module_from_spec(spec)
    argv = sys.argv
    sys.argv = ["bench.py"]
    try:
        spec.loader.exec_module(b)
    finally:
        sys.argv = argv
    out[rank] = b.max_over_ranks(values[rank], dist)
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world_2():
    import torch.multiprocessing as mp
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()  # no fork of a process that may hold CUDA state
    out = mgr.dict()
    mp.spawn(_rank_main, args=(2, port, [12.5, 31.25], out), nprocs=2, join=True)
    assert out[0] == out[1] == 31.25


def test_reference_arm_under_torchrun_world_2():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--workload", "c1", "--gpus", "2", "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
