"""The N>1 path of bench.py on the CPU: world size 2 over gloo.  Images are
independent, so N GPUs run N replicas with no data-path collective; the bench
only needs its barrier and the max over ranks of the timed region, and the
reference arm runs on rank 0 alone."""
import json
import os
import socket
import subprocess
import sys

from conftest import ROOT

HELPERS = r"""
import os, sys
sys.path.insert(0, os.environ["GST_ROOT"])
import bench
rank, world, local = bench.dist_init(2)
assert world == 2 and rank == int(os.environ["RANK"])
bench.barrier(world)
got = bench.max_over_ranks(0.5 + rank, world)   # rank 0: 0.5, rank 1: 1.5
bench.barrier(world)
print("MAX", rank, got, flush=True)
import torch.distributed as dist
dist.destroy_process_group()
"""


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def cpu_env(**extra) -> dict:
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", MASTER_ADDR="127.0.0.1", GST_ROOT=str(ROOT))
    env.update({k: str(v) for k, v in extra.items()})
    return env


def test_barrier_and_max_over_two_gloo_ranks():
    port = free_port()
    procs = [subprocess.Popen([sys.executable, "-c", HELPERS], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                              env=cpu_env(RANK=r, LOCAL_RANK=r, WORLD_SIZE=2, MASTER_PORT=port), text=True)
             for r in range(2)]
    outs = []
    for p in procs:
        out, _ = p.communicate(timeout=300)
        assert p.returncode == 0, out
        outs.append(out)
    got = sorted(line.split()[1:] for out in outs for line in out.splitlines() if line.startswith("MAX"))
    assert got == [["0", "1.5"], ["1", "1.5"]]


def test_reference_arm_under_torchrun_two_ranks():
    # The driver's launch form: rank 0 times the reference's CPU path and
    # prints one line, the other rank exits 0 without work.
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--cpu-sample", "2"]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=cpu_env(), cwd=str(ROOT))
    assert p.returncode == 0, p.stdout + p.stderr
    lines = [json.loads(line) for line in p.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
