"""bench.py's host logic on CPU: the replica path on CPU ranks (gloo, world size 2: the
max-over-ranks time, the whole-job rate, the reference arm's rank > 0 exiting without work)
and the clocks record built from nvidia-smi samples."""
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


def test_clock_sampler_summary():
    """The clocks record of the bench line from nvidia-smi's CSV samples: median SM clock,
    maximum, peak power and the throttle reasons seen active in any sample."""
    import bench

    class Proc:  # stands in for the finished nvidia-smi process
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    cs = bench.ClockSampler(0)
    cs.proc = Proc()
    cs.lines = ["0, 2070, 2070, 610.5, 0x0, Not Active, Not Active, Not Active, Not Active",
                "0, 1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
                "0, 2055, 2070, 700.0, 0x0, Not Active, Not Active, Not Active, Not Active",
                "garbled", "0, [N/A], 2070, 1.0, 0x0, a, b, c, d"]
    out = cs.stop()
    assert out["samples"] == 3 and out["sm_mhz"] == 2055.0 and out["sm_max_mhz"] == 2070.0
    assert out["power_w_max"] == 1390.0 and out["reasons"] == ["sw_power_cap"]
    cs.lines[0] = "0, 1400, 2070, 600.0, 0x40, Not Active, Active, Not Active, Not Active"
    assert bench.ClockSampler.stop(cs)["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    empty = bench.ClockSampler(0)
    assert empty.stop()["reasons"] == ["nvidia-smi unavailable"]


def test_reference_arm_other_ranks_do_nothing(monkeypatch, capsys):
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class A:
        steps, warmup, workload = 3, 3, "simp64"

    assert bench.run_reference(A) is None
    assert capsys.readouterr().out == ""
