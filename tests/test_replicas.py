"""Replicas on several GPUs (bench.py --gpus N): every rank renders its own frames, no
collective on the data path; the job's throughput is all ranks' frames over the slowest
rank's time. Run here as world-size-2 gloo process groups on the CPU."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    out = {"env": bench.dist_init(),
           "max": bench.max_over_ranks(1.5 + rank, "cpu"),
           "rate": bench.job_rate(100, 1.0 + rank, "cpu")}  # rank 1 is the slower replica
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, out))


def test_rates_aggregate_over_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        assert got[r]["env"] == (2, r, r)
        assert got[r]["max"] == 2.5
        assert got[r]["rate"] == pytest.approx(2 * 100 / 2.0)  # both ranks' frames over the slower time


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm's other ranks exit at once, printing nothing."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
