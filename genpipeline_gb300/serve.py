"""Serving loop for FEM solve requests: continuous batching on one GPU.

A request is a forward solve: an edge n (cubic n^3 grid), a density seed and a load case,
usually with its densities as payload (``attach_payloads``; without one the server draws them
from the seed). Load cases are built once per (edge, load). Requests arrive over time. Between two defect-correction rounds of the running batch the
server:
- admits every arrived request for which a slot and device memory are free (free HBM from
  ``torch.cuda.mem_get_info`` minus a reserve);
- retires the designs that finished in the round.

So a request that arrives while others are on the GPU joins the next round, and its work
overlaps theirs inside the same persistent launch (``gbsimp_batch_round``). A finished
request's displacement stays on the device in a warm-start cache keyed by (n, seed, load),
so a repeated design starts from its previous solution. The reference has no serving loop:
its BO evaluates FEM requests through a thread pool with one CSR assembly and one PCG loop
per request (voxel_fem.py:559-611, gpu_fem_solver.py:76-133).
"""
from __future__ import annotations

import collections
import os
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import torch

from . import _lib as L
from . import designs as D
from .batch import BatchFEM, FEMDesign
from .engine import Engine, get_engine, n_dof


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

    @property
    def latency(self) -> float:
        return self.done_at - self.arrival


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
    def __init__(self, engine: Optional[Engine] = None, max_slots: int = 24, memory_reserve: float = 0.1,
                 rtol: float = 1e-8, warm_cache_entries: int = 256, keep_solutions: bool = False):
        self.eng = engine or get_engine()
        self.batch = BatchFEM(self.eng, L.make_law("modified", 3.0), rtol=rtol)
        self.max_slots = max_slots
        self.memory_reserve = memory_reserve
        self.warm = collections.OrderedDict()
        self.warm_entries = warm_cache_entries
        self.keep_solutions = keep_solutions
        self.in_use = 0
        self.rounds = 0
        self.max_active = 0
        self._loads = {}  # (n, load case) -> (f, fixed DOFs) on the host, built once

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
        free, total = torch.cuda.mem_get_info(self.eng.device)
        return need <= free - self.memory_reserve * total

    def _retire(self, d: FEMDesign, now: float):
        r: Request = d.tag
        r.done_at = now
        r.compliance = d.compliance
        r.iterations = d.stats["iterations"]
        r.status = d.stats["status"]
        key = (r.n, r.seed, r.load)
        self.warm[key] = d.du
        self.warm.move_to_end(key)
        while len(self.warm) > self.warm_entries:
            self.warm.popitem(last=False)
        if self.keep_solutions:
            r.u = d.du
        self.in_use -= d.device_bytes(self.eng.lib)
        d.dx = d.df = d.dmask = d.ws = None

    def run(self, requests: List[Request], realtime: bool = True) -> dict:
        """Serves ``requests`` (arrival times relative to the start). With realtime=False all
        requests are available at once (arrival order is kept)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        queue = collections.deque()
        nxt = 0
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        done: List[Request] = []
        while len(done) < len(reqs):
            t = now()
            while nxt < len(reqs) and (not realtime or reqs[nxt].arrival <= t):
                queue.append(reqs[nxt])
                nxt += 1
            # admission: free slots and free device memory
            while queue and len(self.batch.items) < self.max_slots:
                r = queue[0]
                d = self._design(r)
                need = d.device_bytes(self.eng.lib)
                if self.batch.items and not self._fits(need):
                    break
                queue.popleft()
                r.admitted_at = now()
                self.batch.add(d)
                self.in_use += need
            self.max_active = max(self.max_active, len(self.batch.items))
            if self.batch.items:
                finished = self.batch.round()
                self.rounds += 1
                tn = now()
                for d in finished:
                    self._retire(d, tn)
                    done.append(d.tag)
            elif nxt < len(reqs):
                time.sleep(max(0.0, min(0.01, reqs[nxt].arrival - now())))
        lat = np.array([r.latency for r in done])
        span = max(r.done_at for r in done) - min(r.arrival for r in done)
        return {"requests": len(done), "solves_per_s": len(done) / span, "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
                "rounds": self.rounds, "max_active": self.max_active,
                "warm_starts": int(sum(r.warm for r in done)),
                "failed": int(sum(r.status not in (L.GBS_OK,) for r in done)),
                "span_s": span}
