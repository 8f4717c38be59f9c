"""The benchmark's multi-process path on the CPU: two ranks over gloo (torchrun's
environment variables, rendezvous on 127.0.0.1).  The product does not shard, so
N processes run N independent replicas; what the harness itself must get right is
the rendezvous, the barrier, the maximum of the ranks' times, and that only rank 0
prints a line (the reference arm runs on rank 0 alone)."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank, port):
    env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    return env


HELPERS = r"""
import sys
sys.path.insert(0, {root!r})
import bench
world, rank, local = bench.dist_init()
bench.barrier(world)
m = bench.max_over_ranks(world, 3.0 * (rank + 1))
print(world, rank, m, flush=True)
"""


def test_two_rank_rendezvous_barrier_and_max():
    port = _free_port()
    code = HELPERS.format(root=ROOT)
    procs = [subprocess.Popen([sys.executable, "-c", code], env=_env(r, port), stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = [p.communicate(timeout=180) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err
    got = sorted(tuple(o.split()) for o, _ in outs)
    assert got == [("2", "0", "6.0"), ("2", "1", "6.0")]


def test_reference_arm_runs_on_rank_zero_only(oracle):
    """`bench.py --impl reference` under two ranks: rank 0 times its bounded CPU
    sample and prints the one JSON line, rank 1 exits 0 without output."""
    port = _free_port()
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--cpu-seconds", "0.3"]
    procs = [subprocess.Popen(cmd, env=_env(r, port), stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                              cwd=ROOT) for r in range(2)]
    outs = [p.communicate(timeout=600) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err[-2000:]
    lines0 = [l for l in outs[0][0].splitlines() if l.startswith("{")]
    assert len(lines0) == 1
    d = json.loads(lines0[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
    assert not [l for l in outs[1][0].splitlines() if l.strip()]
