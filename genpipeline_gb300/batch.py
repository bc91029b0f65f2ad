"""Batched FEM solves: many designs of different sizes per launch (gbsimp_batch_round).

The reference evaluates designs one at a time: ``VoxelFEMEvaluator.evaluate_batch`` fans
``GPUVoxelFEM.solve`` calls out to a thread pool, and each call assembles its own CSR
matrix and runs its own PCG loop (voxel_fem.py:559-611, gpu_fem_solver.py:76-133). Here a
batch shares the GPU inside one persistent kernel per round. Every design gets a share of
the SMs, its own grid barrier and its own scalars; the FP64 defect correction runs in
lockstep rounds around those launches.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import torch

from . import _lib as L
from . import bcs as B
from .engine import INNER_RTOL, Engine, get_engine, n_dof, n_elem


@dataclass
class FEMDesign:
    """One forward solve: densities, load vector and fixed DOFs on a grid (host or device)."""

    grid: tuple
    x: object  # (n_elem,) densities: numpy, or a float32 device tensor
    f: np.ndarray
    fixed_dofs: np.ndarray
    u0: Optional[torch.Tensor] = None  # warm start (FP64, device)
    tag: object = None
    # device state (filled by BatchFEM)
    dx: Optional[torch.Tensor] = field(default=None, repr=False)
    df: Optional[torch.Tensor] = field(default=None, repr=False)
    dmask: Optional[torch.Tensor] = field(default=None, repr=False)
    du: Optional[torch.Tensor] = field(default=None, repr=False)
    ws: Optional[torch.Tensor] = field(default=None, repr=False)
    stats: Optional[dict] = None
    compliance: Optional[float] = None

    def device_bytes(self, lib=None) -> int:
        lib = lib or L.load()
        nx, ny, nz = self.grid
        return int(lib.gbsimp_solve_ws_bytes(nx, ny, nz)) + 4 * n_elem(self.grid) + 16 * n_dof(self.grid) + \
            n_dof(self.grid) // 3


class BatchFEM:
    """Runs gbsimp_batch_round over a changing set of designs. ``round_iters`` > 0 bounds the
    inner PCG iterations of one round (a solve still running is paused and resumes in the
    next round), so that a serving loop regains control every few milliseconds. With
    ``autotune`` (or a ``tuner``), ``solve_all`` first picks the form, SM shares and designs per
    launch for the batch's grid class (autotune.BatchTuner: every candidate timed once on copies
    of the designs, the choice cached per grid class)."""

    def __init__(self, engine: Optional[Engine] = None, law: Optional[L.Law] = None, rtol: float = 1e-8,
                 inner_rtol: float = INNER_RTOL, max_iter: int = 200000, max_outer: int = 30, fused: bool = True,
                 round_iters: int = 0, autotune: bool = False, tuner=None):
        self.eng = engine or get_engine()
        self.law = law or L.make_law("modified", 3.0)
        self._args = dict(rtol=rtol, inner_rtol=inner_rtol, max_iter=max_iter, max_outer=max_outer)
        self.opts = Engine.opts(rtol=rtol, inner_rtol=inner_rtol, max_iter=max_iter, max_outer=max_outer,
                                fused=int(fused), check_every=int(round_iters))
        self.items: List[FEMDesign] = []
        self._structs = None
        if tuner is None and autotune:
            from .autotune import default_tuner

            tuner = default_tuner()
        self.tuner = tuner
        self.config = None  # the autotune.BatchConfig applied by the last solve_all (None: the options as given)

    def apply_config(self, cfg) -> None:
        """Sets the batch parameters of an autotune.BatchConfig."""
        self.opts.fused = int(cfg.fused)
        self.opts.batch_share = int(cfg.batch_share)
        self.opts.batch_group = int(cfg.batch_group)
        self.config = cfg

    def _trial(self, designs: List[FEMDesign], cfg) -> float:
        """Seconds of one whole solve of copies of `designs` under cfg: the same device densities,
        loads and masks, their warm starts copied, new displacements and workspaces (the designs
        themselves are left as they are)."""
        from .autotune import timed

        bf = BatchFEM(self.eng, self.law, round_iters=int(self.opts.check_every), **self._args)
        bf.apply_config(cfg)
        copies = []
        for d in designs:
            if d.dx is None:
                self.upload(d)
            c = FEMDesign(d.grid, d.x, d.f, d.fixed_dofs, tag=None)
            c.dx, c.df, c.dmask = d.dx, d.df, d.dmask
            c.du = (d.u0.to(device=self.eng.device, dtype=torch.float64).clone() if d.u0 is not None
                    else torch.zeros(n_dof(d.grid), dtype=torch.float64, device=self.eng.device))
            c.ws = torch.empty_like(d.ws)
            copies.append(c)
        out = []
        t = timed(lambda: out.extend(bf._solve_loop(copies)), torch.cuda.synchronize)
        if len(out) != len(copies) or any(c.stats["status"] != L.GBS_OK for c in out):
            raise RuntimeError(f"trial of {cfg} did not solve every design")
        return t

    def upload(self, d: FEMDesign) -> FEMDesign:
        dev = self.eng.device
        nx, ny, nz = d.grid
        if isinstance(d.x, torch.Tensor):  # densities already on the device (e.g. from gbsimp_voxel_prep)
            d.dx = d.x.reshape(-1).to(device=dev, dtype=torch.float32).contiguous()
        else:
            d.dx = torch.as_tensor(np.asarray(d.x, dtype=np.float32).reshape(-1), device=dev).contiguous()
        d.df = torch.as_tensor(np.asarray(d.f, dtype=np.float64), device=dev).contiguous()
        d.dmask = torch.as_tensor(B.node_mask(nx, ny, nz, d.fixed_dofs), device=dev)
        if d.u0 is not None:
            d.du = d.u0.to(device=dev, dtype=torch.float64).clone().contiguous()
        else:
            d.du = torch.zeros(n_dof(d.grid), dtype=torch.float64, device=dev)
        d.ws = torch.empty(int(self.eng.lib.gbsimp_solve_ws_bytes(nx, ny, nz)), dtype=torch.uint8, device=dev)
        return d

    def add(self, d: FEMDesign) -> FEMDesign:
        if d.dx is None:
            self.upload(d)
        d._item = L.BatchItem(d.grid[0], d.grid[1], d.grid[2], 0, d.dx.data_ptr(), d.df.data_ptr(),
                              d.dmask.data_ptr(), d.du.data_ptr(), d.ws.data_ptr(), d.ws.numel(), L.SolveStats())
        self.items.append(d)
        return d

    def round(self) -> List[FEMDesign]:
        """One defect-correction round for every active design; returns the designs that
        finished in it (and drops them from the batch)."""
        if not self.items:
            return []
        arr = (L.BatchItem * len(self.items))(*[d._item for d in self.items])
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        L.check(self.eng.lib.gbsimp_batch_round(self.eng.ctx, arr, len(self.items), C.byref(self.law),
                                                C.byref(self.opts), stream))
        done, keep = [], []
        for i, d in enumerate(self.items):
            d._item = arr[i]
            if arr[i].state != 0:
                d.stats = arr[i].stats.as_dict()
                d.compliance = float(torch.dot(d.df, d.du).item())
                done.append(d)
            else:
                keep.append(d)
        self.items = keep
        return done

    def remove(self, d: FEMDesign) -> bool:
        """Drops a design between rounds (a cancelled request); its inner solve, paused or not,
        is abandoned. Returns False when it is not in the batch."""
        for i, e in enumerate(self.items):
            if e is d:
                del self.items[i]
                return True
        return False

    def solve_all(self, designs: List[FEMDesign]) -> List[FEMDesign]:
        if self.tuner is not None and designs:
            for d in designs:
                if d.dx is None:
                    self.upload(d)
            self.apply_config(self.tuner.tune([d.grid for d in designs], lambda cfg: self._trial(designs, cfg)))
        return self._solve_loop(designs)

    def _solve_loop(self, designs: List[FEMDesign]) -> List[FEMDesign]:
        for d in designs:
            self.add(d)
        out = []
        # each item ends within max_outer FP64 rounds; a round budget adds rounds per correction
        per = 1 if self.opts.check_every <= 0 else 1 + int(self.opts.max_iter) // int(self.opts.check_every)
        for _ in range((int(self.opts.max_outer) + 2) * per):
            out += self.round()
            if not self.items:
                break
        return out


class SolveQueue:
    """The native solve queue (gbsimp_queue_*): designs are submitted at any time, each poll
    runs one defect-correction round for everything queued (the persistent batched PCG
    inside) and hands back the designs that finished. The same continuous batching as
    BatchFEM, with the queue kept by the library."""

    def __init__(self, engine: Optional[Engine] = None, law: Optional[L.Law] = None, rtol: float = 1e-8,
                 inner_rtol: float = INNER_RTOL, max_iter: int = 200000, max_outer: int = 30, fused: bool = True,
                 round_iters: int = 0):
        self.eng = engine or get_engine()
        self.law = law or L.make_law("modified", 3.0)
        self.opts = Engine.opts(rtol=rtol, inner_rtol=inner_rtol, max_iter=max_iter, max_outer=max_outer,
                                fused=int(fused), check_every=int(round_iters))
        h = C.c_void_p()
        L.check(self.eng.lib.gbsimp_queue_create(self.eng.ctx, C.byref(self.law), C.byref(self.opts), C.byref(h)))
        self._q = h
        self._by_addr = {}  # address of a submitted item struct -> its design (keeps the struct alive)
        self._uploader = BatchFEM(self.eng, self.law)

    def submit(self, d: FEMDesign) -> FEMDesign:
        if d.dx is None:
            self._uploader.upload(d)
        d._qitem = L.BatchItem(d.grid[0], d.grid[1], d.grid[2], 0, d.dx.data_ptr(), d.df.data_ptr(),
                               d.dmask.data_ptr(), d.du.data_ptr(), d.ws.data_ptr(), d.ws.numel(), L.SolveStats())
        L.check(self.eng.lib.gbsimp_queue_submit(self._q, C.byref(d._qitem)))
        self._by_addr[C.addressof(d._qitem)] = d
        return d

    def poll(self, max_done: int = 64) -> List[FEMDesign]:
        arr = (C.POINTER(L.BatchItem) * max_done)()
        n = C.c_int()
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        L.check(self.eng.lib.gbsimp_queue_poll(self._q, arr, max_done, C.byref(n), stream))
        out = []
        for k in range(n.value):
            d = self._by_addr.pop(C.addressof(arr[k].contents))
            d.stats = d._qitem.stats.as_dict()
            d.compliance = float(torch.dot(d.df, d.du).item())
            out.append(d)
        return out

    def __len__(self) -> int:
        return int(self.eng.lib.gbsimp_queue_size(self._q))

    def close(self):
        if self._q:
            self.eng.lib.gbsimp_queue_destroy(self._q)
            self._q = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_plain(designs: List[FEMDesign], engine: Optional[Engine] = None, law: Optional[L.Law] = None,
                rtol: float = 1e-8, inner_rtol: float = INNER_RTOL) -> List[FEMDesign]:
    """The one-design-at-a-time form: one gbsimp_solve (graph-loop PCG) per design."""
    eng = engine or get_engine()
    law = law or L.make_law("modified", 3.0)
    bf = BatchFEM(eng, law)
    for d in designs:
        if d.dx is None:
            bf.upload(d)
        d.stats = eng.solve(d.grid, law, d.dx, d.df, d.dmask, d.du, rtol=rtol, inner_rtol=inner_rtol,
                            key=f"plain:{d.grid}")
        d.compliance = float(torch.dot(d.df, d.du).item())
    return designs
