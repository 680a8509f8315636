"""The N > 1 harness of bench.py on CPU: two gloo ranks.

bench.py runs one replica per rank (the path has no exchange step); what the
ranks share is the harness: process-group start-up, the barrier around the
timed region, the max-over-ranks time and rank-0-only output.  These tests run
that harness with world_size 2 on the gloo backend, and the reference arm under
torch.distributed.run, where rank 0 alone works and prints.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _harness_rank(rank, world, port, out_dir):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    w, r, local = bench.dist_init(None)
    assert (w, r, local) == (world, rank, rank)
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    # each rank reports its own time; the harness keeps the slowest
    t = bench.allmax(w, 1.5 + rank)
    bench.barrier(w)
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"rank": r, "max": t}, f)
    dist.destroy_process_group()


def test_harness_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_harness_rank, args=(world, free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn", join=True)
    got = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(world)]
    assert [g["rank"] for g in got] == [0, 1]
    assert all(g["max"] == 2.5 for g in got)


def test_reference_arm_under_torchrun_prints_once():
    pytest.importorskip("torch")
    env = dict(os.environ)
    env.pop("CUDA_VISIBLE_DEVICES", None)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["n_gpus"] == 2 and line["steps"] == 2
    assert line["value"] > 0 and line["unit"] == "pairs/s"
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
