"""FEMServer's host logic without a GPU: admission by free memory, refusal of a request that
can never fit, queueing behind running designs, and cancellation of queued and running
requests. The batch is a host stand-in that finishes a design after a fixed number of rounds;
the failure records follow the reference's sentinel convention (voxel_fem.py:270-298)."""
import numpy as np

from genpipeline_gb300.pipeline_utils import FEM_SENTINEL
from genpipeline_gb300.serve import FEMServer, Request


class FakeBatch:
    """Stands in for BatchFEM: a design of edge n finishes after n // 8 rounds."""

    def __init__(self, on_round=None):
        self.items = []
        self.left = {}
        self.on_round = on_round
        self.rounds = 0

    def add(self, d):
        self.items.append(d)
        self.left[id(d)] = max(1, d.grid[0] // 8)

    def remove(self, d):
        if d in self.items:
            self.items.remove(d)
            return True
        return False

    def round(self):
        self.rounds += 1
        if self.on_round:
            self.on_round(self)
        done = []
        for d in list(self.items):
            self.left[id(d)] -= 1
            if self.left[id(d)] == 0:
                d.stats = {"status": 0, "iterations": 10 * d.grid[0]}
                d.compliance = float(d.grid[0])
                done.append(d)
                self.items.remove(d)
        return done


def _reqs(edges):
    return [Request(i, 0.0, n, i, "cantilever") for i, n in enumerate(edges)]


def _server(batch, capacity, **kw):
    """A device of `capacity` bytes: free memory shrinks as designs are admitted (16 bytes per
    element)."""
    srv = None

    def mem_info():
        return capacity - srv.in_use, capacity

    srv = FEMServer(batch=batch, mem_info=mem_info, bytes_of=lambda d: 16 * int(np.prod(d.grid)),
                    memory_reserve=0.0, **kw)
    return srv


def test_request_larger_than_the_device_is_refused_with_the_sentinel_record():
    reqs = _reqs([8, 24, 8, 16])
    srv = _server(FakeBatch(), capacity=16 * 20 ** 3)  # 24^3 can never fit, 16^3 can
    s = srv.run(reqs, realtime=False)
    assert s["requests"] == 4 and s["refused"] == 1 and s["solved"] == 3
    big = reqs[1]
    assert big.failure_reason == "no_memory" and big.compliance == FEM_SENTINEL
    assert big.result() == {"compliance": FEM_SENTINEL, "failure_reason": "no_memory"}
    assert all(r.failure_reason is None and r.compliance == r.n for r in reqs if r.n != 24)
    assert srv.in_use == 0


def test_requests_wait_for_memory_held_by_running_designs():
    reqs = _reqs([16] * 6)
    srv = _server(FakeBatch(), capacity=2 * 16 * 16 ** 3 + 100)  # two 16^3 designs at a time
    s = srv.run(reqs, realtime=False)
    assert s["solved"] == 6 and s["refused"] == 0
    assert s["max_active"] == 2
    assert s["rounds"] == 3 * 2  # three waves of two designs, two rounds each
    assert all(r.admitted_at is not None for r in reqs)


def test_lower_reserve_admits_more_at_once():
    reqs = _reqs([16] * 6)
    cap = 4 * 16 * 16 ** 3
    tight = _server(FakeBatch(), capacity=cap)
    tight.memory_reserve = 0.5  # half the device kept free: two designs at a time
    a = tight.run(reqs, realtime=False)
    loose = _server(FakeBatch(), capacity=cap)
    b = loose.run(_reqs([16] * 6), realtime=False)
    assert a["max_active"] == 2 and b["max_active"] == 4 and a["rounds"] > b["rounds"]


def test_cancel_queued_and_running_requests():
    reqs = _reqs([24, 24, 16, 8, 8])
    srv = None

    def on_round(batch):
        if batch.rounds == 1:  # another thread cancels while the first round runs
            srv.cancel(0)  # running (admitted first)
            srv.cancel(4)  # still queued (one slot left after the first admissions)
            srv.cancel(99)  # unknown: ignored

    srv = _server(FakeBatch(on_round), capacity=10 ** 9, max_slots=3)
    s = srv.run(reqs, realtime=False)
    assert s["requests"] == 5 and s["cancelled"] == 2 and s["solved"] == 3
    assert reqs[0].failure_reason == "cancelled" and reqs[0].compliance == FEM_SENTINEL
    assert reqs[4].failure_reason == "cancelled" and reqs[4].admitted_at is None
    assert [r.failure_reason for r in reqs[1:4]] == [None, None, None]
    assert srv.in_use == 0 and not srv.batch.items
