"""``SIMPSolver`` with the interface and semantics of genpipeline/topology/simp_solver.py.

Same constructor (nx, ny, nz, penal, rmin, boundary_conditions, preserved_mask), same
``run(volfrac, n_iters, force_mag) -> (nx, ny, nz) ndarray`` and ``last_compliance``, same
stiffness law ``max(x, 1e-3)^penal`` (:182-185), boundary conditions (:81-175), filter
(:1545-1567) and OC bisection (:225-249). The loop runs on the GPU: each OC iteration is
one FP32-inner/FP64-outer solve to rtol 1e-8 (the reference solves directly with spsolve,
:192), the element sensitivities, the filter chain rule and the bisection, all on the device.

The reference's element table (:284-1543) is not symmetric positive semi-definite, which
conjugate gradients need; ``Ke`` here is the SPD 2x2x2-Gauss stiffness of the same
element (E = 1, nu = 0.3).
"""
from __future__ import annotations

import numpy as np

from .. import _lib as L
from .. import bcs as B
from ..engine import Engine
from ..simp import SimpProblem, SolveSpec


class SIMPSolver:
    def __init__(self, nx: int = 32, ny: int = 8, nz: int = 8, penal: float = 3.0, rmin: float = 1.5,
                 boundary_conditions: dict | None = None, preserved_mask: np.ndarray | None = None):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.penal = penal
        self.rmin = rmin
        self.Ke = Engine.ke_quadrature(0.3, 1.0)
        self.last_compliance = 0.0
        self.preserved_mask = None if preserved_mask is None else np.asarray(preserved_mask).flatten().astype(bool)
        self.bcs = {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2}
        if boundary_conditions:
            self.bcs.update(boundary_conditions)
        self.rtol = 1e-8
        self.last_run = None

    def _get_bcs(self, force_mag: float):
        """(f, fixed_dofs) exactly as simp_solver.py:81-157."""
        return B.reference_cpu(self.nx, self.ny, self.nz, self.bcs, force_mag)

    def run(self, volfrac: float = 0.4, n_iters: int = 80, force_mag: float = 1.0) -> np.ndarray:
        f, fixed = self._get_bcs(force_mag)
        spec = SolveSpec(grid=(self.nx, self.ny, self.nz), penal=self.penal, rmin=self.rmin, volfrac=volfrac,
                         law="ref", oc_variant=dict(L.OC_CPU), rtol=self.rtol)
        prob = SimpProblem(spec, f, fixed, preserved=self.preserved_mask)
        for i in range(n_iters):
            st = prob.step()
            if st["status"] not in (L.GBS_OK, L.GBS_ENOTCONV):
                raise L.GbsimpError(st["status"], f"SIMP solve failed at iteration {i}: {st}")
            if (i + 1) % 10 == 0:
                print(f"  [SIMP] Iter {i + 1:3d} | Mean xPhys: {float(prob.xphys.mean()):.3f}")
        self.last_compliance = prob.final_compliance()
        self.last_run = prob
        return prob.xphys_numpy()
