"""The modal kernels for 168 <= nz <= 446: three 16-byte groups per thread and plane, row
lengths set at run time (for nz <= 167 the kernels use two groups and compile-time row
lengths; nz = 167 is that form's largest plane, checked here too). Same checks and
tolerances as the small-grid parity tests: the FP32 apply within
2e-6 of max|y| and the FP64 apply within 1e-12 of the FP64 oracle, with and without the
Dirichlet mask; a refined solve's compliance within 1e-6 of the oracle's FP64 PCG.

This file sorts after every other test, so that a run stopping at its first failure has run
them all.
"""
import numpy as np
import pytest
import torch

from genpipeline_gb300 import _lib as L
from genpipeline_gb300 import bcs
from genpipeline_gb300.engine import Engine, n_dof, n_elem
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MAT = O.Material("modified", 3.0, emin=1e-9)


@pytest.fixture(scope="module")
def eng():
    return Engine()


def _cuda(a, dtype=None):
    t = torch.as_tensor(np.ascontiguousarray(a)).cuda()
    return t if dtype is None else t.to(dtype)


@pytest.mark.parametrize("grid", [(4, 3, 167), (4, 3, 168), (3, 5, 300), (2, 2, 446)])
@pytest.mark.parametrize("masked", [False, True])
def test_tall_z_apply_vs_oracle(eng, grid, masked):
    rng = np.random.default_rng(sum(grid) + masked)
    x = rng.uniform(0.0, 1.0, n_elem(grid)).astype(np.float32)
    x[:3] = [0.0, 5e-4, 1.0]
    p = rng.standard_normal(n_dof(grid))
    fixed = bcs.reference_cpu(*grid, {"fixed_face": ["x_min", "z_max"]})[1] if masked else None
    ref = O.apply(grid, O.ke_quadrature(), O.moduli(x.astype(np.float64), MAT), p,
                  bcs.dof_mask(*grid, fixed) if masked else None)
    law = L.make_law("modified", 3.0)
    m = _cuda(bcs.node_mask(*grid, fixed)) if masked else None
    assert eng.apply_path(grid[2]) == "modal"
    y32 = eng.apply(grid, law, _cuda(x), _cuda(p, torch.float32), m).cpu().numpy()
    np.testing.assert_allclose(y32, ref, rtol=0, atol=2e-6 * np.abs(ref).max())
    y64 = eng.apply(grid, law, _cuda(x), _cuda(p), m).cpu().numpy()
    np.testing.assert_allclose(y64, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("grid", [(8, 4, 200), (3, 2, 446)])
def test_tall_z_refined_solve_vs_oracle(eng, grid):
    f, fixed = bcs.LOAD_CASES["cantilever"](*grid)
    x = np.random.default_rng(5).uniform(0.05, 1.0, n_elem(grid)).astype(np.float32)
    dm = bcs.dof_mask(*grid, fixed)
    uref, _, _ = O.pcg(grid, O.ke_quadrature(), O.moduli(x.astype(np.float64), MAT), f, dm, tol=1e-13)
    u = torch.zeros(n_dof(grid), dtype=torch.float64, device="cuda")
    st = eng.solve(grid, L.make_law("modified", 3.0), _cuda(x), _cuda(f), _cuda(bcs.node_mask(*grid, fixed)), u,
                   rtol=1e-8)
    assert st["status"] == L.GBS_OK and st["relres"] <= 1e-8, st
    ug = u.cpu().numpy()
    assert float(f @ ug) == pytest.approx(float(f @ uref), rel=1e-6)
    np.testing.assert_allclose(ug, uref, rtol=0, atol=1e-5 * np.abs(uref).max())
