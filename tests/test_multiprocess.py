"""The N > 1 path of bench.py on the CPU: two gloo ranks on 127.0.0.1.

The path does not shard (each rank renders the whole workload as a replica,
"scaling": "weak"), so its only multi-rank logic is on the host: each
timing's maximum over the ranks, the whole-job rate from it, and the
reference arm, which rank 0 alone runs.  The same functions run over NCCL on
GPUs; here gloo carries the collective.
"""
import contextlib
import io
import os
import socket
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        mine = [[1.0, 5.0], [3.0, 2.0]][rank]
        ms = bench.max_over_ranks(mine, world, torch.device("cpu"))
        rate = bench.job_rate(1000, world, ms[0])
        with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
            f.write(f"{ms[0]} {ms[1]} {rate}\n")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_replica():
    import torch.multiprocessing as mp
    world = 2
    with tempfile.TemporaryDirectory() as d:
        mp.spawn(_rank_main, args=(world, _free_port(), d), nprocs=world, join=True)
        lines = [open(os.path.join(d, f"rank{r}.txt")).read().split() for r in range(world)]
    for vals in lines:
        a, b, rate = (float(v) for v in vals)
        assert (a, b) == (3.0, 5.0)  # element-wise maximum over the ranks
        assert rate == pytest.approx(1000 * world / 3e-3)


def test_single_rank_needs_no_process_group():
    import torch
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([2.5, 4.0], 1, torch.device("cpu")) == [2.5, 4.0]
    assert bench.job_rate(10, 1, 2.0) == pytest.approx(5000.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"])
    args = bench.parse()
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(args)
    assert buf.getvalue() == ""  # rank 1 exits without work or output
