"""The replica path of bench.py (one process per GPU, torchrun's environment)
on two CPU ranks over gloo: rendezvous on 127.0.0.1, the barrier, the
max-over-ranks timing, and the reference arm's rank-0-only run."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def run_ranks(code, world=2, timeout=120):
    port = str(free_port())
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=port, CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", code], cwd=ROOT, env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=timeout)
        assert p.returncode == 0, err[-2000:]
        outs.append(out)
    return outs


def test_two_ranks_rendezvous_barrier_and_max_over_ranks():
    code = (
        "import json, sys\n"
        "sys.path.insert(0, '.')\n"
        "import bench\n"
        "rank, world = bench.dist_setup(2)\n"
        "slowest = bench.reduce_max(0.010 * (rank + 1), world)\n"
        "bench.barrier(world)\n"
        "print(json.dumps({'rank': rank, 'world': world, 'slowest': slowest}))\n")
    outs = [json.loads(o.strip().splitlines()[-1]) for o in run_ranks(code)]
    assert sorted(o["rank"] for o in outs) == [0, 1]
    assert all(o["world"] == 2 for o in outs)
    # every rank sees the slowest replica's time, so value = units of all
    # ranks / that time is the same figure everywhere
    assert all(abs(o["slowest"] - 0.020) < 1e-12 for o in outs)


def test_reference_arm_runs_on_rank_zero_only():
    # rank 1 of `bench.py --impl reference --gpus 2` returns at once: no work, no line
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2", MASTER_ADDR="127.0.0.1", MASTER_PORT="1",
               CUDA_VISIBLE_DEVICES="")
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""
