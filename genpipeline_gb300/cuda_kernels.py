"""The SIMP kernel functions of genpipeline/cuda_kernels/__init__.py on the GB300 library.

Same names, signatures and results:
- ``simp_sensitivity`` and ``simp_sensitivity_aggressive`` (:286-326, :475-502):
  dc_e = -penal * max(x_e, 1e-3)^(penal-1) * u_e^T Ke u_e over an arbitrary element -> DOF
  table ``edof_mat``;
- ``fused_spmv`` (:329-368): y = sum_e max(x_e, 1e-3)^penal * P_e^T Ke P_e p;
- ``pcg_solve_cuda`` (:443-473): Jacobi-PCG on a CSR matrix with a fixed-DOF list.

The reference falls back to Python loops when its extension fails (:310-324); this module has
no fallback and raises instead. Inputs may be float32/float64 and int32/int64; the results
follow the dtype of ``xPhys`` (or ``b``).
"""
from __future__ import annotations

import hashlib

import numpy as np
import torch

from . import _lib as L
from .engine import Engine

__all__ = ["simp_sensitivity", "simp_sensitivity_aggressive", "fused_spmv", "pcg_solve_cuda"]

_ENGINES: dict = {}


def _engine_for(Ke: torch.Tensor, device: torch.device) -> Engine:
    """One library context per (device, element stiffness): Ke travels as a kernel argument."""
    k = np.ascontiguousarray(Ke.detach().to(torch.float64).cpu().numpy().reshape(24, 24))
    key = (device.index, hashlib.sha1(k.tobytes()).hexdigest())
    e = _ENGINES.get(key)
    if e is None:
        e = Engine(device, ke=k)
        _ENGINES[key] = e
    return e


def _check(xPhys, Ke, edof_mat):
    if not (xPhys.is_cuda and edof_mat.is_cuda):
        raise RuntimeError("genpipeline_gb300.cuda_kernels needs CUDA tensors (no CPU fallback)")
    if Ke.numel() != 576:
        raise ValueError("Ke must be 24x24")
    if edof_mat.dim() != 2 or edof_mat.shape[1] != 24:
        raise ValueError("edof_mat must be (n_elem, 24)")


def simp_sensitivity(xPhys: torch.Tensor, u: torch.Tensor, Ke: torch.Tensor, edof_mat: torch.Tensor, penal: float,
                     nx: int, ny: int, nz: int) -> torch.Tensor:
    _check(xPhys, Ke, edof_mat)
    eng = _engine_for(Ke, xPhys.device)
    x = xPhys.reshape(-1).to(torch.float32).contiguous()
    uf = u.reshape(-1).to(torch.float32).contiguous()
    edof = edof_mat if edof_mat.dtype in (torch.int32, torch.int64) else edof_mat.to(torch.int64)
    dc = eng.sensitivity_edof(L.make_law("ref", penal), x, uf, edof.contiguous())
    return dc.to(xPhys.dtype).reshape(xPhys.shape)


def simp_sensitivity_aggressive(xPhys: torch.Tensor, u: torch.Tensor, Ke: torch.Tensor, edof_mat: torch.Tensor,
                                penal: float, nx: int, ny: int, nz: int) -> torch.Tensor:
    """Same result as ``simp_sensitivity`` (the reference intends the two to agree to 1%)."""
    return simp_sensitivity(xPhys, u, Ke, edof_mat, penal, nx, ny, nz)


def fused_spmv(xPhys: torch.Tensor, p: torch.Tensor, Ke: torch.Tensor, edof_mat: torch.Tensor, penal: float,
               nx: int, ny: int, nz: int) -> torch.Tensor:
    _check(xPhys, Ke, edof_mat)
    eng = _engine_for(Ke, xPhys.device)
    x = xPhys.reshape(-1).to(torch.float32).contiguous()
    pf = p.reshape(-1).to(torch.float32).contiguous()
    edof = edof_mat if edof_mat.dtype in (torch.int32, torch.int64) else edof_mat.to(torch.int64)
    y = eng.apply_edof(L.make_law("ref", penal), x, pf, edof.contiguous())
    return y.to(p.dtype).reshape(p.shape)


def pcg_solve_cuda(row_ptr: torch.Tensor, col_idx: torch.Tensor, values: torch.Tensor, diagonal: torch.Tensor,
                   b: torch.Tensor, x0: torch.Tensor, fixed_dofs: torch.Tensor, max_iter: int = 100,
                   tol: float = 1e-6) -> torch.Tensor:
    if not b.is_cuda:
        raise RuntimeError("pcg_solve_cuda needs CUDA tensors (no CPU fallback)")
    eng = _engine_for(torch.as_tensor(Engine.ke_quadrature()), b.device)
    x = x0.reshape(-1).to(torch.float32).clone().contiguous()
    fixed = None
    if fixed_dofs is not None and fixed_dofs.numel() > 0:
        fixed = fixed_dofs.reshape(-1).to(torch.int32).contiguous()
    eng.pcg_csr(row_ptr.to(torch.int32).contiguous(), col_idx.to(torch.int32).contiguous(),
                values.to(torch.float32).contiguous(), diagonal.reshape(-1).to(torch.float32).contiguous(),
                b.reshape(-1).to(torch.float32).contiguous(), x, fixed, rtol=float(tol), max_iter=int(max_iter))
    return x.to(b.dtype).reshape(b.shape)
