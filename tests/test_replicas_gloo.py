"""Replicas (bench.py under torchrun, one process per GPU): the ranks run
disjoint frame pairs, the job's time is the slowest rank's (one all-reduce,
the only cross-rank traffic), the reported value counts every rank's pairs,
and the reference arm's other ranks exit without work.  Two gloo processes
on the CPU stand in for the ranks."""
import os
import pathlib
import socket
import subprocess
import sys

import pytest

REPO = pathlib.Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, str(REPO))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    frames = bench.rank_frames(rank, 3)
    t = bench.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
    value = bench.job_value(world, 3, 4, t)
    everyone = [None] * world
    dist.all_gather_object(everyone, frames)
    dist.destroy_process_group()
    q.put((rank, t, value, everyone))


def test_two_ranks_split_pairs_and_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, value, everyone in out:
        assert t == 15.0  # the slower rank's time
        assert value == pytest.approx(2 * 3 * 4 / 0.015)
        assert set(everyone[0]).isdisjoint(everyone[1])
        assert sorted(everyone[0] + everyone[1]) == list(range(6))


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--gpus",
                        "2", "--steps", "1", "--warmup", "0"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
