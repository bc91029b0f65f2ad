"""``GPUVoxelFEM`` with the interface and semantics of genpipeline/fem/gpu_fem_solver.py.

It does one forward solve on a voxel grid (penal = 1, so K is proportional to the densities
floored at 1e-3), with the face-distributed load of ``SIMPSolverGPU._get_bcs``. The solve
uses tol = 1e-3 with 200 iterations, as the reference does (:96); grids below 50,000 DOFs,
which the reference factorises directly, are solved to 1e-10 (``SIMPSolverGPU._solve``). It returns
``{"stress_max", "displacement_max", "compliance"}`` with the reference's proxies and its
sentinel for near-void designs (:122-133). ``GPUConjugateGradientFEM`` is kept as an alias
(:137).
"""
from __future__ import annotations

import logging

import numpy as np
import torch

from ..topology.simp_solver_gpu import SIMPSolverGPU

logger = logging.getLogger(__name__)

_VOXEL_SIZE_M = 0.001


class GPUVoxelFEM:
    def __init__(self, voxels: np.ndarray, fixed_face: str = "x_min", load_face: str = "x_max", load_dof: int = 2,
                 force_n: float = 1000.0, device: str = "cuda"):
        nx, ny, nz = voxels.shape
        self._device = device
        self._voxels_flat = torch.from_numpy(np.asarray(voxels).flatten().astype(np.float32)).to("cuda")
        self._force_n = force_n
        bcs = {"fixed_face": fixed_face, "load_face": load_face, "load_dof": load_dof}
        self._simp = SIMPSolverGPU(nx=nx, ny=ny, nz=nz, penal=1.0, rmin=1.5, boundary_conditions=bcs,
                                   device="cuda", dtype=torch.float32)

    def solve(self) -> dict:
        simp = self._simp
        K = simp._assemble_K(self._voxels_flat)
        f, fixed_dofs = simp._get_bcs(self._force_n)
        u = simp._solve(K, f, fixed_dofs, tol=1e-3, max_iter=200)
        compliance = float(torch.dot(u, f).item())
        u_np = u.detach().cpu().numpy()
        disp_abs = float(np.linalg.norm(u_np.reshape(-1, 3), axis=1).max())
        disp_max_mm = float(np.clip(disp_abs * _VOXEL_SIZE_M * 1e3, 0, 1e4))
        n_solid = int((self._voxels_flat > 0.5).sum().item())
        if n_solid < 50 or not np.isfinite(compliance) or compliance < 1.0:
            return {"stress_max": 1e4, "displacement_max": 1e3, "compliance": 1e6}
        stress = float(np.clip(compliance / max(n_solid, 1) * 10.0, 0, 1e4))
        return {"stress_max": stress, "displacement_max": disp_max_mm,
                "compliance": float(np.clip(compliance, 0, 1e8))}


GPUConjugateGradientFEM = GPUVoxelFEM
