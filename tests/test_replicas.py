"""Replicas runs (bench.py under torchrun, one process per GPU, no collective
on the data path): the timing reduction over ranks and the reference arm's
rank-0-only rule, with two gloo ranks on the CPU (127.0.0.1)."""

import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import json, os, sys
sys.path.insert(0, os.environ["KPT_ROOT"])
import torch.distributed as dist
dist.init_process_group("gloo")
import bench
rank, world, _ = bench.env_rank()
ms = bench.max_over_ranks(10.0 + 5.0 * rank, world)
# every rank sees the slowest rank's time; whole-job throughput counts every
# rank's units over it
value = 100.0 * world / ms
dist.barrier()
dist.destroy_process_group()
print(json.dumps({"rank": rank, "world": world, "ms": ms, "value": value}))
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _launch(code, world, extra_env=None):
    port = _free_port()
    procs = []
    for rank in range(world):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                   WORLD_SIZE=str(world), LOCAL_RANK=str(rank), KPT_ROOT=ROOT, **(extra_env or {}))
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err
        outs.append(out)
    return outs


def test_timing_is_the_slowest_rank_and_value_counts_every_rank():
    outs = [json.loads(o.strip().splitlines()[-1]) for o in _launch(WORKER, 2)]
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["world"] == 2 and o["ms"] == 15.0
        assert abs(o["value"] - 200.0 / 15.0) < 1e-12


def test_one_rank_keeps_its_own_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5


def test_reference_arm_runs_on_rank_0_only():
    """Under torchrun the reference arm prints one line from rank 0; the
    other ranks exit 0 without work (rank 1 alone here: it must print
    nothing and return at once)."""
    code = ("import os, sys; sys.path.insert(0, os.environ['KPT_ROOT']); import bench, argparse; "
            "bench.run_reference(argparse.Namespace(gpus=2, steps=1, warmup=0))")
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", KPT_ROOT=ROOT)
    p = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""
