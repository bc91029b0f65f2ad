"""The replica path of bench.py on CPU ranks (gloo, world size 2): the max-over-ranks time,
the whole-job rate, and the reference arm's rank > 0 exiting without work."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, out):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(times[rank], world, "cpu")
    out[rank] = (t, bench.whole_job_rate(world, 10, t))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_rate():
    world, port = 2, _free_port()
    times = [1.25, 2.5]
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank_main, args=(world, port, times, out), nprocs=world, start_method="spawn")
        res = dict(out)
    assert res[0] == res[1] == (2.5, 2 * 10 / 2.5)


def test_single_rank_rate():
    import bench

    assert bench.max_over_ranks(3.0, 1, "cpu") == 3.0
    assert bench.whole_job_rate(1, 6, 3.0) == 2.0


def test_reference_arm_other_ranks_do_nothing(monkeypatch, capsys):
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class A:
        steps, warmup, workload = 3, 3, "simp64"

    assert bench.run_reference(A) is None
    assert capsys.readouterr().out == ""
