"""Device-resident SIMP loop (one OC iteration = solve, sensitivity, filter chain rule, OC).

The sequence is the reference loop of genpipeline/topology/simp_solver.py:56-79:
    dc = _sensitivity(xPhys)        solve K(xPhys) u = f, ce = u_e^T Ke u_e, dc = -E'(xPhys) ce
    dc = _filter_dc(dc)             dc <- H^T (dc / Hs)
    x, xPhys = _oc_update(...)      bisection on the multiplier, xPhys = H xnew / Hs
and after the loop a final solve gives the compliance f.u. Densities, displacements (the
warm start of the next solve) and every intermediate stay in HBM; the host only reads the
solver status.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import torch

from . import _lib as L
from . import bcs as B
from .engine import INNER_RTOL, Engine, get_engine, n_dof, n_elem


@dataclass
class SolveSpec:
    """Knobs of one SIMP problem (the reference's constructor arguments plus precision)."""

    grid: tuple
    penal: float = 3.0
    rmin: float = 1.5
    volfrac: float = 0.3
    law: str = "ref"            # "ref": max(x,1e-3)^p (simp_solver.py:182-185); "modified": Emin + x^p (E0-Emin)
    e0: float = 1.0
    emin: float = 1e-9
    xmin: float = 1e-3
    oc_variant: dict = field(default_factory=lambda: dict(L.OC_CPU))
    rtol: float = 1e-8          # FP64 outer residual target
    inner_rtol: float = INNER_RTOL  # FP32 PCG reduction per outer correction (engine.INNER_RTOL)
    max_iter: int = 200000
    max_outer: int = 30
    fused: bool = False         # persistent one-launch PCG (grid barriers) instead of the graph loop
    # warm start of solve k >= 3: u_{k-1} + warm_theta (u_{k-1} - u_{k-2}) (0: u_{k-1}); the value
    # of the native loop (gbsimp_simp_run), whose designs this loop reproduces bit for bit
    warm_theta: float = 0.5
    # 1: the outer residual's element products in FP64 (default: double-float FP32 pairs, whose
    # rounding is below 1e-12 ||D f||; the FP64 u, the norms and the compliance are FP64 either way)
    residual_fp64: bool = False

    def material(self) -> L.Law:
        return L.make_law(self.law, self.penal, self.e0, self.emin, self.xmin)


class SimpProblem:
    """One SIMP design on the device."""

    def __init__(self, spec: SolveSpec, f: np.ndarray, fixed_dofs: np.ndarray,
                 preserved: Optional[np.ndarray] = None, engine: Optional[Engine] = None,
                 x_init: Optional[np.ndarray] = None, device=None):
        self.spec = spec
        self.grid = tuple(int(v) for v in spec.grid)
        self.eng = engine if engine is not None else get_engine(device)
        dev = self.eng.device
        nx, ny, nz = self.grid
        ne, nd = n_elem(self.grid), n_dof(self.grid)
        self.law = spec.material()
        self.f = torch.as_tensor(np.asarray(f, dtype=np.float64), device=dev).contiguous()
        if self.f.numel() != nd:
            raise ValueError(f"load vector has {self.f.numel()} entries, expected {nd}")
        self.fixed_dofs = np.asarray(fixed_dofs, dtype=np.int64)
        self.mask = torch.as_tensor(B.node_mask(nx, ny, nz, self.fixed_dofs), device=dev)
        self.pres = None
        if preserved is not None:
            p = np.asarray(preserved).reshape(-1).astype(bool)
            if p.size != ne:
                raise ValueError("preserved mask size mismatch")
            self.pres = torch.as_tensor(p.astype(np.uint8), device=dev)
        if x_init is None:
            x0 = np.full(ne, spec.volfrac, dtype=np.float32)
        else:
            x0 = np.asarray(x_init, dtype=np.float32).reshape(-1)
        self.x = torch.as_tensor(x0, device=dev).contiguous()
        if self.pres is not None:
            self.x[self.pres.bool()] = 1.0
        self.xphys = self.x.clone()
        self.u = torch.zeros(nd, dtype=torch.float64, device=dev)
        self.u_prev = torch.zeros(nd, dtype=torch.float64, device=dev)
        self.solved = 0  # solutions of this loop held in u (and u_prev)
        self.dc = torch.empty(ne, dtype=torch.float32, device=dev)
        self.dcf = torch.empty(ne, dtype=torch.float32, device=dev)
        self.xnew = torch.empty(ne, dtype=torch.float32, device=dev)
        self.energy = torch.zeros((), dtype=torch.float64, device=dev)
        self.comp = torch.zeros((), dtype=torch.float64, device=dev)
        self.hs = self.eng.filter_hs(self.grid, spec.rmin)
        self._oc_key = f"oc:{id(self)}"
        self.eng.oc_prepare(self.grid, spec.rmin, self.pres, key=self._oc_key)
        self.iteration = 0
        self.history = []

    # ---- pieces ----------------------------------------------------------------------
    profile = False  # time the PCG apply launches with CUDA events (reported in the stats)

    def solve(self, rtol: Optional[float] = None) -> dict:
        s = self.spec
        return self.eng.solve(self.grid, self.law, self.xphys, self.f, self.mask, self.u,
                              rtol=s.rtol if rtol is None else rtol, inner_rtol=s.inner_rtol,
                              max_iter=s.max_iter, max_outer=s.max_outer, key=f"solve:{id(self)}",
                              profile=self.profile, fused=s.fused, residual_fp64=s.residual_fp64)

    def step(self) -> dict:
        """One OC iteration of the reference loop."""
        s = self.spec
        if s.warm_theta > 0.0 and self.solved >= 2:
            self.eng.warm_start(self.u, self.u_prev, s.warm_theta)
        elif self.solved == 1:
            self.u_prev.copy_(self.u)
        st = self.solve()
        self.solved += 1
        self.eng.sensitivity(self.grid, self.law, self.xphys, self.u, dc=self.dc, energy=self.energy)
        self.eng.filter(self.grid, s.rmin, self.dc, hs=self.hs, transpose=True, out=self.dcf)
        self.eng.oc(self.grid, s.rmin, s.volfrac, self.x, self.dcf, self.pres, s.oc_variant, xnew=self.xnew,
                    xphys=self.xphys, key=self._oc_key, prepared=True)
        self.x, self.xnew = self.xnew, self.x
        self.iteration += 1
        self.history.append(st)
        return st

    def state(self):
        """A copy of the loop's state (design, xPhys, displacements and the warm-start history)."""
        return (self.x.clone(), self.xphys.clone(), self.u.clone(), self.u_prev.clone(), self.solved)

    def restore(self, state) -> None:
        x, xphys, u, u_prev, solved = state
        self.x.copy_(x)
        self.xphys.copy_(xphys)
        self.u.copy_(u)
        self.u_prev.copy_(u_prev)
        self.solved = solved

    def save_state(self, path: str) -> None:
        """Writes what the next iterations depend on to an .npz file: the design x, xPhys, the
        displacements of the last two solves (the warm start) and the iteration counters. The
        reference keeps a SIMP run's state in memory only (simp_solver_gpu.py:65,793); with
        load_state a run can resume in another process and continue bit for bit."""
        with open(path, "wb") as fh:  # the file is `path` itself (np.savez would append .npz to a name)
            np.savez(fh, x=self.x.cpu().numpy(), xphys=self.xphys.cpu().numpy(), u=self.u.cpu().numpy(),
                     u_prev=self.u_prev.cpu().numpy(), solved=np.int64(self.solved),
                     iteration=np.int64(self.iteration), grid=np.asarray(self.grid, dtype=np.int64))

    def load_state(self, path: str) -> None:
        """Restores a state written by save_state into this problem (same grid; the load case,
        material and solve settings are this problem's own)."""
        with np.load(path) as d:
            if tuple(int(v) for v in d["grid"]) != self.grid:
                raise ValueError(f"state of grid {tuple(d['grid'])} does not fit grid {self.grid}")
            self.restore((torch.as_tensor(d["x"]), torch.as_tensor(d["xphys"]), torch.as_tensor(d["u"]),
                          torch.as_tensor(d["u_prev"]), int(d["solved"])))
            self.iteration = int(d["iteration"])

    def compliance(self) -> float:
        """f . u of the current displacement (synchronises)."""
        self.eng.dot64(self.f, self.u, out=self.comp)
        return float(self.comp.item())

    def final_compliance(self) -> float:
        """SIMPSolver.run's closing solve on the final xPhys (simp_solver.py:78)."""
        self.solve()
        return self.compliance()

    def run(self, n_iters: int) -> np.ndarray:
        for _ in range(n_iters):
            st = self.step()
            if st["status"] not in (L.GBS_OK, L.GBS_ENOTCONV):
                raise L.GbsimpError(st["status"], f"solve failed at iteration {self.iteration}: {st}")
        return self.xphys_numpy()

    def xphys_numpy(self) -> np.ndarray:
        return self.xphys.detach().cpu().numpy().astype(np.float64).reshape(self.grid)
