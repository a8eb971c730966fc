"""The multi-process path of bench.py on CPU (gloo, world size 2): the
process-group set-up, barrier and max-over-ranks timing the replicas use,
and the reference arm's rule that only rank 0 measures. The GPU path has no
collective in its data path (shots are independent replicas)."""
import os
import socket
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys, types
sys.path.insert(0, {repo!r})
import bench
args = types.SimpleNamespace()
world, rank, local = bench.dist_setup(args)
assert world == 2 and rank == int(os.environ["RANK"])
bench.barrier(world)
m = bench.max_over_ranks(1.5 + rank, world)
assert m == 2.5, m
if rank == 1:
    # the reference arm: ranks other than 0 exit without work
    ra = types.SimpleNamespace(n=8, nt=4, steps=1, warmup=0, snap="bf16")
    assert bench.run_reference(ra) == 0
import torch.distributed as dist
dist.destroy_process_group()
print("ok", rank)
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_gloo_helpers():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(repo=REPO)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    outs = [p.communicate(timeout=240)[0] for p in procs]
    for rank, (p, out) in enumerate(zip(procs, outs)):
        assert p.returncode == 0, out
        assert f"ok {rank}" in out, out


def test_gpus_flag_launches_replicas_without_torchrun():
    """`bench.py --gpus 2` outside torchrun starts two replica processes
    itself (torch.distributed.run on 127.0.0.1, gloo here) and rank 0 prints
    one line with the max over both ranks."""
    import json
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    env["CUDA_VISIBLE_DEVICES"] = ""
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--gpus", "2", "--dry-run"], env=env,
                       capture_output=True, text=True, timeout=240)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["dry_run"] and d["n_gpus"] == 2 and d["max_rank_seconds"] >= 0.02
