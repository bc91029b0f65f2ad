"""``DenseGPUSolver`` with the interface of genpipeline/topology/simp_solver_dense_gpu.py.

The constructor (nx, ny, nz, penal, rmin, device), ``run(volfrac=0.25, n_iters=15,
force_mag=1000)`` and ``last_compliance`` are kept, and so are the class's boundary
conditions. Those fix the x_min, y_min and z_min faces and spread a -z load over every
node of the x_max face (:209-236). The class's OC is the CPU-style bisection (:371-391) and
its PCG tolerance is 1e-5 with 500 iterations (:330-357).

The reference assembles a dense n_dof x n_dof matrix (O(n_dof^2): 7.8 GB at 32x16x16) from
a made-up element table (:104-138). Here the same loop runs matrix-free on the SPD
hexahedron stiffness, so only the interface and the boundary conditions are reproduced; the
reference's numbers are not a parity target.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _lib as L
from .. import bcs as B
from ..simp import SimpProblem, SolveSpec


class DenseGPUSolver:
    def __init__(self, nx: int = 32, ny: int = 8, nz: int = 8, penal: float = 3.0, rmin: float = 1.5,
                 device: str = "cuda"):
        if not torch.cuda.is_available():
            raise RuntimeError("DenseGPUSolver needs a CUDA GPU (no CPU fallback)")
        self.nx, self.ny, self.nz = nx, ny, nz
        self.penal = penal
        self.rmin = rmin
        self.device = device
        self.n_elem = nx * ny * nz
        self.n_nodes = (nx + 1) * (ny + 1) * (nz + 1)
        self.n_dof = 3 * self.n_nodes
        self.last_compliance = 0.0
        self.use_cuda_kernels = True

    def _get_bcs(self, force_mag: float):
        return B.reference_dense(self.nx, self.ny, self.nz, force_mag)

    def run(self, volfrac: float = 0.25, n_iters: int = 15, force_mag: float = 1000) -> np.ndarray:
        f, fixed = self._get_bcs(force_mag)
        spec = SolveSpec(grid=(self.nx, self.ny, self.nz), penal=self.penal, rmin=self.rmin, volfrac=volfrac,
                         law="ref", oc_variant=dict(L.OC_CPU), rtol=1e-5, max_iter=500)
        prob = SimpProblem(spec, f, fixed)
        for i in range(n_iters):
            prob.step()
            self.last_compliance = prob.compliance()
            if (i + 1) % 5 == 0:
                print(f"  [DenseGPU] Iter {i + 1:3d} | Mean: {prob.xphys.mean().item():.3f} | "
                      f"Max: {prob.xphys.max().item():.3f}", flush=True)
        return prob.xphys_numpy()
