"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

The solve path does not shard: under torchrun each rank runs an independent
replica of the workload, and the job's time is the slowest rank's.  These
tests run that reduction and the reference arm's rank gating as real
processes, without a GPU.
"""
import json
import os
import socket
import subprocess
import sys
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import json, os, sys
sys.path.insert(0, os.environ["BENCH_ROOT"])
import torch.distributed as dist
import bench
rank, local, world = bench.dist_env()
dist.init_process_group("gloo")
t = bench.max_over_ranks(1.5 + rank, world, device="cpu")
dist.barrier()
print(json.dumps({"rank": rank, "world": world, "t": t, "rate": bench.job_rate(world, 5, t)}), flush=True)
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank, world, port):
    env = dict(os.environ)
    env.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(port), BENCH_ROOT=ROOT, CUDA_VISIBLE_DEVICES="")
    return env


def test_max_over_ranks_gloo():
    port = _free_port()
    procs = [subprocess.Popen([sys.executable, "-c", WORKER], env=_env(r, 2, port), stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["world"] == 2
        assert o["t"] == 2.5                 # the slower rank's time, on every rank
        assert o["rate"] == 2 * 5 / 2.5      # both ranks' steps over that time
    assert sorted(o["rank"] for o in outs) == [0, 1]


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(0.75, 1) == 0.75
    assert bench.job_rate(1, 3, 0.75) == 4.0


def test_reference_arm_runs_on_rank0_only():
    """Under torchrun the reference arm's other ranks exit 0 at once, printing nothing."""
    t0 = time.time()
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=_env(1, 2, _free_port()), capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
    assert time.time() - t0 < 60
