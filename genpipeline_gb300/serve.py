"""Serving loop for FEM solve requests: continuous batching on one GPU.

A request is a forward solve: an edge n (cubic n^3 grid), a density seed and a load case,
usually with its densities as payload (``attach_payloads``; without one the server draws them
from the seed). Load cases are built once per (edge, load). Requests arrive over time. A round
of the running batch runs at most ``round_iters`` inner PCG iterations per design (a solve
still running is paused on the device and resumes in the next round), so rounds last a few
milliseconds whatever the grid sizes. Between two rounds the server:
- drops cancelled requests (``cancel``), queued or running;
- admits every arrived request for which a slot and device memory are free (free HBM from
  ``torch.cuda.mem_get_info`` minus a reserve); a request that does not fit even when nothing
  else is on the device is refused at once;
- retires the designs that finished in the round.

So a request that arrives while others are on the GPU joins within one round, and its work
overlaps theirs inside the same persistent launch (``gbsimp_batch_round``). A finished
request's displacement stays on the device in a warm-start cache keyed by (n, seed, load),
so a repeated design starts from its previous solution. Refused and cancelled requests get the
reference's failure record: every output FEM_SENTINEL and a ``failure_reason``
(voxel_fem.py:270-298, pipeline_utils.py:18-33). The reference has no serving loop: its BO
evaluates FEM requests through a thread pool with one CSR assembly and one PCG loop per
request (voxel_fem.py:559-611, gpu_fem_solver.py:76-133).
"""
from __future__ import annotations

import collections
import os
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import Callable, List, Optional

import numpy as np
import torch

from . import _lib as L
from . import designs as D
from .batch import BatchFEM, FEMDesign
from .engine import Engine, get_engine, n_dof
from .pipeline_utils import FEM_SENTINEL


@dataclass
class Request:
    rid: int
    arrival: float  # seconds after the start of the stream
    n: int
    seed: int
    load: str
    repeat: bool = False
    # the client's payload: the (n, n, n) FP32 densities (None: the server draws them from
    # `seed` with designs.grf_density)
    density: Optional[np.ndarray] = field(default=None, repr=False)
    # results
    admitted_at: Optional[float] = None
    done_at: Optional[float] = None
    compliance: Optional[float] = None
    iterations: Optional[int] = None
    status: Optional[int] = None
    warm: bool = False
    u: Optional[torch.Tensor] = field(default=None, repr=False)
    # None for a solved request; "no_memory" (refused at admission), "cancelled" or
    # "solve_failed" (the solver's status is in `status`), with compliance = FEM_SENTINEL
    failure_reason: Optional[str] = None

    @property
    def latency(self) -> float:
        return self.done_at - self.arrival

    def result(self) -> dict:
        """The reference's evaluation record: the outputs, or FEM_SENTINEL everywhere and the
        failure reason (voxel_fem.py:270-298)."""
        if self.failure_reason is not None:
            return {"compliance": FEM_SENTINEL, "failure_reason": self.failure_reason}
        return {"compliance": self.compliance}


def request_stream(n_requests: int = 2000, rate: float = 200.0, edges=(24, 32, 48, 64, 96), repeat_frac: float = 0.1,
                   seed: int = 12345) -> List[Request]:
    """Poisson arrivals at ``rate`` (exponential inter-arrival times), edge ~ U(edges), load
    ~ U(cantilever, top patch, torsion), density seed = request id; about ``repeat_frac`` of
    the requests repeat an earlier (design, load) pair. One PCG64(seed) generator."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out: List[Request] = []
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate)
        if out and rng.random() < repeat_frac:
            j = int(rng.integers(0, len(out)))
            src = out[j]
            out.append(Request(i, t, src.n, src.seed, src.load, repeat=True))
        else:
            n = int(edges[int(rng.integers(0, len(edges)))])
            load = D.LOADS[int(rng.integers(0, len(D.LOADS)))]
            out.append(Request(i, t, n, i, load))
    return out


def attach_payloads(requests: List[Request], workers: Optional[int] = None) -> List[Request]:
    """Gives every request its density payload (designs.grf_density of its edge and seed), as
    a client that sends the design with the request would; repeated designs share one array.
    The fields are drawn on a thread pool (numpy's FFT and generators release the GIL; each
    field has its own seeded generator, so the arrays do not depend on the pool). Returns the
    same list."""
    keys = list(dict.fromkeys((r.n, r.seed) for r in requests))
    with ThreadPoolExecutor(max_workers=workers or os.cpu_count() or 1) as ex:
        made = dict(zip(keys, ex.map(lambda k: D.grf_density((k[0], k[0], k[0]), k[1]), keys)))
    for r in requests:
        r.density = made[(r.n, r.seed)]
    return requests


class FEMServer:
    """``batch`` (default: a BatchFEM on ``engine``) and ``mem_info`` (default:
    torch.cuda.mem_get_info of the engine's device, returning (free, total) bytes) can be
    replaced, e.g. by host-only stand-ins that exercise admission, refusal and cancellation
    without a GPU. ``bytes_of(design)`` gives a design's device footprint."""

    def __init__(self, engine: Optional[Engine] = None, max_slots: int = 24, memory_reserve: float = 0.1,
                 rtol: float = 1e-8, warm_cache_entries: int = 256, keep_solutions: bool = False,
                 round_iters: int = 256, batch=None, mem_info: Optional[Callable[[], tuple]] = None,
                 bytes_of: Optional[Callable[[FEMDesign], int]] = None):
        self.eng = engine if engine is not None or batch is not None else get_engine()
        self.batch = batch if batch is not None else BatchFEM(self.eng, L.make_law("modified", 3.0), rtol=rtol,
                                                              round_iters=round_iters)
        self.mem_info = mem_info if mem_info is not None else (lambda: torch.cuda.mem_get_info(self.eng.device))
        self.bytes_of = bytes_of if bytes_of is not None else (lambda d: d.device_bytes(L.load()))
        self.max_slots = max_slots
        self.memory_reserve = memory_reserve
        self.warm = collections.OrderedDict()
        self.warm_entries = warm_cache_entries
        self.keep_solutions = keep_solutions
        self.in_use = 0
        self.rounds = 0
        self.max_active = 0
        self._loads = {}  # (n, load case) -> (f, fixed DOFs) on the host, built once
        self._cancel_lock = threading.Lock()
        self._cancelled = set()  # request ids to drop at the next check

    def cancel(self, rid: int) -> None:
        """Cancels request ``rid`` (from any thread): it is dropped before the next round,
        whether it is still queued or already on the device, and finishes with
        failure_reason "cancelled". Cancelling a finished or unknown request does nothing."""
        with self._cancel_lock:
            self._cancelled.add(int(rid))

    def _take_cancelled(self) -> set:
        with self._cancel_lock:
            out, self._cancelled = self._cancelled, set()
        return out

    def _design(self, r: Request) -> FEMDesign:
        grid = (r.n, r.n, r.n)
        key = (r.n, r.load)
        if key not in self._loads:
            self._loads[key] = D.load_case(r.load, r.n)
        f, fixed = self._loads[key]
        u0 = self.warm.get((r.n, r.seed, r.load))
        r.warm = u0 is not None
        x = r.density if r.density is not None else D.grf_density(grid, r.seed)
        return FEMDesign(grid, x, f, fixed, u0=u0, tag=r)

    def _fits(self, need: int) -> bool:
        free, total = self.mem_info()
        return need <= free - self.memory_reserve * total

    def _retire(self, d: FEMDesign, now: float, reason: Optional[str] = None):
        r: Request = d.tag
        r.done_at = now
        self.in_use -= self.bytes_of(d)
        if reason is None:
            r.compliance = d.compliance
            r.iterations = d.stats["iterations"]
            r.status = d.stats["status"]
            if r.status != L.GBS_OK:
                reason = "solve_failed"
            else:
                key = (r.n, r.seed, r.load)
                self.warm[key] = d.du
                self.warm.move_to_end(key)
                while len(self.warm) > self.warm_entries:
                    self.warm.popitem(last=False)
                if self.keep_solutions:
                    r.u = d.du
        if reason is not None:
            r.failure_reason = reason
            r.compliance = FEM_SENTINEL
        d.dx = d.df = d.dmask = d.ws = None

    @staticmethod
    def _fail(r: Request, now: float, reason: str):
        r.done_at = now
        r.failure_reason = reason
        r.compliance = FEM_SENTINEL

    def run(self, requests: List[Request], realtime: bool = True) -> dict:
        """Serves ``requests`` (arrival times relative to the start). With realtime=False all
        requests are available at once (arrival order is kept)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        queue = collections.deque()
        nxt = 0
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        done: List[Request] = []
        running = {}  # request id -> its design in the batch
        while len(done) < len(reqs):
            t = now()
            while nxt < len(reqs) and (not realtime or reqs[nxt].arrival <= t):
                queue.append(reqs[nxt])
                nxt += 1
            # cancellations: queued requests leave the queue, running ones the batch
            cancelled = self._take_cancelled()
            if cancelled:
                keep = collections.deque()
                for r in queue:
                    if r.rid in cancelled:
                        self._fail(r, now(), "cancelled")
                        done.append(r)
                    else:
                        keep.append(r)
                queue = keep
                for rid in cancelled & set(running):
                    d = running.pop(rid)
                    self.batch.remove(d)
                    self._retire(d, now(), "cancelled")
                    done.append(d.tag)
                # requests not arrived yet are cancelled when they arrive
                with self._cancel_lock:
                    self._cancelled |= {rid for rid in cancelled if any(r.rid == rid for r in reqs[nxt:])}
            # admission: free slots and free device memory; a request that cannot fit even on
            # an otherwise empty device is refused instead of waiting forever
            while queue and len(self.batch.items) < self.max_slots:
                r = queue[0]
                d = r.__dict__.get("_design") or self._design(r)
                r._design = d  # a request waiting for memory keeps its host-side design
                need = self.bytes_of(d)
                if not self._fits(need):
                    if self.batch.items:
                        break  # wait for running designs to free memory
                    queue.popleft()
                    self._fail(r, now(), "no_memory")
                    done.append(r)
                    continue
                queue.popleft()
                r.admitted_at = now()
                self.batch.add(d)
                running[r.rid] = d
                self.in_use += need
            self.max_active = max(self.max_active, len(self.batch.items))
            if self.batch.items:
                finished = self.batch.round()
                self.rounds += 1
                tn = now()
                for d in finished:
                    running.pop(d.tag.rid, None)
                    self._retire(d, tn)
                    done.append(d.tag)
            elif nxt < len(reqs):
                time.sleep(max(0.0, min(0.01, reqs[nxt].arrival - now())))
        return self.summary(done)

    def summary(self, done: List[Request]) -> dict:
        solved = [r for r in done if r.failure_reason is None]
        lat = np.array([r.latency for r in solved]) if solved else np.zeros(1)
        span = max(r.done_at for r in done) - min(r.arrival for r in done) if done else 0.0
        return {"requests": len(done), "solved": len(solved),
                "solves_per_s": len(solved) / span if span > 0 else 0.0,
                "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "mean_ms": float(lat.mean() * 1e3), "rounds": self.rounds, "max_active": self.max_active,
                "warm_starts": int(sum(r.warm for r in solved)),
                "failed": int(sum(r.failure_reason == "solve_failed" for r in done)),
                "refused": int(sum(r.failure_reason == "no_memory" for r in done)),
                "cancelled": int(sum(r.failure_reason == "cancelled" for r in done)),
                "span_s": span}
