"""The multi-rank path of bench.py on CPU: two gloo ranks, each a replica of
the single-GPU step. The step does not shard, so the only exchange is the
timing: the job's duration is the maximum over ranks and its rate counts
every rank's particles. The reference arm runs on rank 0 alone."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local = [1.25, 2.5][rank]
    seconds = bench.job_seconds(local, world, "cpu")
    rate = bench.job_rate(65536, 10, world, seconds)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, seconds, rate))


def test_job_time_is_the_slowest_rank_and_rate_counts_every_rank():
    ctx = mp.get_context("spawn")
    out = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(out.get() for _ in range(2))
    for rank, seconds, rate in got:
        assert seconds == 2.5
        assert rate == pytest.approx(65536 * 10 * 2 / 2.5)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_seconds(0.75, 1, "cpu") == 0.75
    assert bench.job_rate(1000, 4, 1, 2.0) == 2000.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = bench.parse_args(["--impl", "reference", "--gpus", "2"])
    assert bench.run_reference_arm(args) == 0
    assert capsys.readouterr().out == ""
