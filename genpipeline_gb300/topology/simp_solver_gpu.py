"""``SIMPSolverGPU`` with the interface and semantics of genpipeline/topology/simp_solver_gpu.py.

Kept from the reference:
- the constructor and ``run(volfrac, n_iters, force_mag, x_init)`` (:16-136);
- the ``x_init`` rescaling, the per-iteration tolerance schedule, the NaN stop and the
  early stop after three iterations with compliance change < 1%;
- the boundary conditions of this class (:138-311): distributed, multi-position and grid
  loads;
- the floored law ``max(x, 1e-3)^penal``;
- the GPU OC variant (:801-841);
- ``last_compliance`` (a fresh solve every iteration, as :111 does);
- the internals the FEM evaluator calls: ``_assemble_K``, ``_get_bcs``, ``_solve``.

Nothing is assembled. ``_assemble_K`` returns a matrix-free operator handle and ``_solve``
runs the library's PCG on it. That PCG is FP32 inside an FP64 defect correction, to the
reference's relative tolerance, warm-started from the previous displacement as ``_u_prev``
is (:793). Below 50,000 DOFs the reference factorises K directly whatever the tolerance
(:581-588), so there the solve runs to 1e-10.
"""
from __future__ import annotations

import pickle
from dataclasses import dataclass

import numpy as np
import torch

from .. import _lib as L
from .. import bcs as B
from ..engine import Engine, get_engine, n_dof, n_elem
from .batch_simp import DIRECT_BELOW, DIRECT_RTOL, reference_schedule


@dataclass
class MatrixFreeK:
    """What ``_assemble_K`` returns: the densities defining K(x), applied on the fly."""

    xphys: torch.Tensor
    law: L.Law
    grid: tuple

    @property
    def shape(self):
        nd = n_dof(self.grid)
        return (nd, nd)


class _BcCache:
    """The boundary conditions of one (grid, boundary_conditions, force) on the device, and the
    node mask of the last fixed-DOF set seen. The reference rebuilds both on the host twice per
    SIMP iteration (its sensitivity solve and its compliance solve), which at 64^3 costs about
    8 ms per build against about 6 ms of device work per iteration."""

    def __init__(self, grid, device):
        self.grid = tuple(grid)
        self.device = device
        self._key = None
        self._f = self._fixed = None
        self._mask_fixed = self._mask = None

    def bcs(self, bcs: dict, force_mag: float):
        """Copies of the cached (f FP64, fixed_dofs int64), rebuilt when `bcs` or the force
        changes (the caller gets tensors of its own, as from a fresh build)."""
        try:
            key = (float(force_mag), pickle.dumps(sorted(bcs.items())))
        except Exception:  # values that cannot be compared: build every call
            key = None
        if key is None or key != self._key:
            f, fixed = B.reference_gpu(*self.grid, bcs, force_mag)
            self._f = torch.as_tensor(f, dtype=torch.float64, device=self.device)
            self._fixed = torch.as_tensor(fixed, dtype=torch.int64, device=self.device)
            self._key = key
        return self._f.clone(), self._fixed.clone()

    def mask(self, fixed_dofs) -> torch.Tensor:
        """Per-node Dirichlet bits of `fixed_dofs`, rebuilt only when the set differs from the
        last one (compared on the device)."""
        fd = torch.as_tensor(fixed_dofs, device=self.device).reshape(-1).to(torch.int64)
        if self._mask is None or not torch.equal(self._mask_fixed, fd):
            self._mask = torch.as_tensor(B.node_mask(*self.grid, fd.detach().cpu().numpy()), device=self.device)
            self._mask_fixed = fd.clone()
        return self._mask


class SIMPSolverGPU:
    _RESOURCE_CACHE = {}
    # (tol, max_iter) of the sensitivity solve per iteration (simp_solver_gpu.py:92-99)
    tol_schedule = staticmethod(reference_schedule)
    # The reference's _solve factorises K directly (SuperLU) whenever the grid has fewer DOFs
    # than this, whatever tolerance it is given (simp_solver_gpu.py:581-588): those solves run
    # here to DIRECT_RTOL, so small grids follow the exact-solve trajectory as the reference's do.
    DIRECT_BELOW = DIRECT_BELOW
    DIRECT_RTOL = DIRECT_RTOL

    def __init__(self, nx: int = 32, ny: int = 8, nz: int = 8, penal: float = 3.0, rmin: float = 1.5,
                 boundary_conditions: dict | None = None, device: str = "cuda",
                 preserved_mask: np.ndarray | None = None, dtype: torch.dtype = torch.float32):
        if not torch.cuda.is_available():
            raise RuntimeError("SIMPSolverGPU needs a CUDA GPU (no CPU fallback)")
        self.nx, self.ny, self.nz = nx, ny, nz
        self.grid = (nx, ny, nz)
        self.penal = penal
        self.rmin = rmin
        self.device = torch.device(device if str(device).startswith("cuda") else "cuda")
        self.dtype = dtype
        self.eng: Engine = get_engine(self.device)
        self.Ke = torch.as_tensor(self.eng.get_ke(), dtype=torch.float64, device=self.device).to(
            torch.float32 if dtype not in (torch.float64,) else torch.float64)
        key = (nx, ny, nz, rmin, str(self.device))
        if key not in SIMPSolverGPU._RESOURCE_CACHE:
            SIMPSolverGPU._RESOURCE_CACHE[key] = {"Hs": self.eng.filter_hs(self.grid, rmin)}
        self._Hs = SIMPSolverGPU._RESOURCE_CACHE[key]["Hs"]
        self.last_compliance = 0.0
        self.preserved_mask = None
        if preserved_mask is not None:
            self.preserved_mask = torch.as_tensor(np.asarray(preserved_mask).flatten().astype(np.uint8),
                                                  device=self.device)
        self.bcs = {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2}
        if boundary_conditions:
            self.bcs.update(boundary_conditions)
        self._bc_cache = _BcCache(self.grid, self.device)
        self._u_prev = None
        self._law = L.make_law("ref", penal)
        self._oc_key = f"ocgpu:{id(self)}"
        self._oc_ready = False
        self.history = []

    # ---- internals with the reference's names -------------------------------------------
    def _get_bcs(self, force_mag: float):
        """(f, fixed_dofs) as device tensors, simp_solver_gpu.py:138-248 (built once per
        boundary conditions and force, then copied on the device)."""
        return self._bc_cache.bcs(self.bcs, force_mag)

    def _assemble_K(self, xPhys: torch.Tensor) -> MatrixFreeK:
        x = torch.as_tensor(xPhys, device=self.device).reshape(-1).to(torch.float32).contiguous()
        return MatrixFreeK(x, L.make_law("ref", self.penal), self.grid)

    def _mask(self, fixed_dofs: torch.Tensor) -> torch.Tensor:
        return self._bc_cache.mask(fixed_dofs)

    def _solve(self, K: MatrixFreeK, f: torch.Tensor, fixed_dofs: torch.Tensor, tol: float = 1e-6,
               max_iter: int = 2000, x0: torch.Tensor | None = None) -> torch.Tensor:
        """u with K(x) u = f on the free DOFs to relative residual ``tol`` (at most
        ``max_iter`` PCG iterations; the best iterate is returned when the cap is hit, as the
        reference's loop does). Grids below ``DIRECT_BELOW`` DOFs are solved to
        ``DIRECT_RTOL`` instead, the accuracy of the reference's direct solve there."""
        if n_dof(K.grid) < self.DIRECT_BELOW:
            tol, max_iter = self.DIRECT_RTOL, 1000000
        ff = torch.as_tensor(f, device=self.device).reshape(-1).to(torch.float64).contiguous()
        u = torch.zeros_like(ff) if x0 is None else torch.as_tensor(x0, device=self.device).reshape(-1).to(
            torch.float64).clone()
        st = self.eng.solve(K.grid, K.law, K.xphys, ff, self._mask(fixed_dofs), u, rtol=float(tol),
                            max_iter=int(max_iter), key=f"solve:{id(self)}")
        self.last_solve = st
        if st["status"] not in (L.GBS_OK, L.GBS_ENOTCONV):
            u.fill_(float("nan"))
        self._u_prev = u.clone()
        return u

    def _calculate_compliance(self, xPhys: torch.Tensor, force_mag: float) -> float:
        f, fixed = self._get_bcs(force_mag)
        u = self._solve(self._assemble_K(xPhys), f, fixed)
        return float(torch.dot(f, u).item())

    def _sensitivity(self, xPhys: torch.Tensor, force_mag: float, tol: float = 1e-6, max_iter: int = 300):
        f, fixed = self._get_bcs(force_mag)
        K = self._assemble_K(xPhys)
        u = self._solve(K, f, fixed, tol=tol, max_iter=max_iter, x0=self._u_prev)
        dc = self.eng.sensitivity(self.grid, self._law, K.xphys, u)
        self._u_prev = u
        return dc

    def _filter_dc(self, dc: torch.Tensor) -> torch.Tensor:
        d = torch.as_tensor(dc, device=self.device).reshape(-1).to(torch.float32).contiguous()
        return self.eng.filter(self.grid, self.rmin, d, hs=self._Hs, transpose=True)

    def _oc_update(self, x: torch.Tensor, xPhys: torch.Tensor, dc: torch.Tensor, volfrac: float):
        """GPU variant of the bisection (simp_solver_gpu.py:801-841)."""
        xf = torch.as_tensor(x, device=self.device).reshape(-1).to(torch.float32).contiguous()
        dcf = torch.as_tensor(dc, device=self.device).reshape(-1).to(torch.float32).contiguous()
        if not self._oc_ready:
            self.eng.oc_prepare(self.grid, self.rmin, self.preserved_mask, key=self._oc_key)
            self._oc_ready = True
        return self.eng.oc(self.grid, self.rmin, volfrac, xf, dcf, self.preserved_mask, L.OC_GPU,
                           key=self._oc_key, prepared=True)

    # ---- the loop -----------------------------------------------------------------------
    def run(self, volfrac: float = 0.4, n_iters: int = 15, force_mag: float = 1.0,
            x_init: np.ndarray | None = None) -> np.ndarray:
        ne = n_elem(self.grid)
        if x_init is not None:
            x = torch.as_tensor(np.asarray(x_init).flatten(), device=self.device).to(torch.float32)
            x = x * (volfrac / x.mean().clamp(min=1e-6))
            x = x.clamp(1e-3, 1.0)
        else:
            x = torch.full((ne,), float(volfrac), device=self.device, dtype=torch.float32)
        if self.preserved_mask is not None:
            x[self.preserved_mask.bool()] = 1.0
        x = x.contiguous()
        xPhys = x.clone()
        prev = float("inf")
        changes = []
        change = 0.0
        curr = float("nan")
        for i in range(n_iters):
            tol, max_iter = self.tol_schedule(i)
            dc = self._sensitivity(xPhys, force_mag, tol=tol, max_iter=max_iter)
            if torch.isnan(dc).any():
                print(f"  [SIMP-GPU] FATAL: NaN in sensitivity at iter {i}")
                break
            dc = self._filter_dc(dc)
            x, xPhys = self._oc_update(x, xPhys, dc, volfrac)
            curr = self._calculate_compliance(xPhys, force_mag)
            self.history.append(curr)
            if prev != float("inf"):
                change = abs(prev - curr) / (prev + 1e-10)
                changes.append(change)
            if len(changes) >= 3 and all(c < 0.01 for c in changes[-3:]):
                print(f"  [SIMP-GPU] Early stop at iter {i + 1} (converged, change={change:.2%})")
                break
            prev = curr
            if (i + 1) % 5 == 0 or i == n_iters - 1:
                print(f"  [SIMP-GPU] Iter {i + 1:3d} | Mean: {xPhys.mean().item():.3f} | "
                      f"Max: {xPhys.max().item():.3f} | dC: {change:.2%}")
        self.last_compliance = curr
        return xPhys.reshape(self.nx, self.ny, self.nz).cpu().numpy()
