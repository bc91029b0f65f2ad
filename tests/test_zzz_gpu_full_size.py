"""Parity at the full benchmark sizes: 64^3 (262,144 elements) and 192x96x96 (1,769,472
elements, 5,447,811 DOFs).

- The FP32 and FP64 applies against the FP64 oracle's apply on the same seeded inputs (the
  oracle's matrix-free apply takes about 0.1 s at 192x96x96 on the host cores). The FP32
  error of one output is set by the sums of at most 8 elements x 24 terms that form it, so the
  bound does not grow with the grid: the small-grid tolerance of 2e-6 of max|y| holds per
  output, checked here as 1e-6 in relative 2-norm and 6e-6 of max|y| at the worst output (the
  extra factor covers the tail of 5.4 million outputs instead of tens of thousands).
- A refined solve at 192x96x96 (the edge line load, seeded densities U(0.05, 1)) checked
  independently of the solver's own residual: the oracle's dense FP64 apply gives
  ||D(f - K u)|| <= 1.5e-8 ||D f||. Its energy u.K.u from the sensitivity kernel matches
  the compliance f.u to within |u.r| <= ||u|| ||r|| (1e-5 relative).

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

FULL = [(64, 64, 64), (192, 96, 96)]


@pytest.fixture(scope="module")
def eng():
    return Engine()


def _cuda(a, dtype=None):
    t = torch.as_tensor(np.ascontiguousarray(a)).cuda()
    return t if dtype is None else t.to(dtype)


@pytest.mark.parametrize("grid", FULL)
@pytest.mark.parametrize("masked", [False, True])
def test_full_size_apply_vs_oracle(eng, grid, masked):
    rng = np.random.default_rng(hash((grid, masked)) % 2**32)
    x = rng.uniform(0.0, 1.0, n_elem(grid)).astype(np.float32)
    x[:3] = [0.0, 5e-4, 1.0]
    p = rng.standard_normal(n_dof(grid))
    fixed = bcs.LOAD_CASES["edge_line"](*grid)[1] if masked else None
    ref = O.apply(grid, O.ke_quadrature(), O.moduli(x.astype(np.float64), O.Material("modified", 3.0, emin=1e-9)),
                  p, bcs.dof_mask(*grid, fixed) if masked else None)
    law = L.make_law("modified", 3.0)
    m = _cuda(bcs.node_mask(*grid, fixed)) if masked else None
    assert eng.apply_path(grid[2]) == "modal"
    y32 = eng.apply(grid, law, _cuda(x), _cuda(p, torch.float32), m).cpu().numpy().astype(np.float64)
    scale = np.abs(ref).max()
    assert np.linalg.norm(y32 - ref) <= 1e-6 * np.linalg.norm(ref)
    assert np.abs(y32 - ref).max() <= 6e-6 * scale
    y64 = eng.apply(grid, law, _cuda(x), _cuda(p), m).cpu().numpy()
    np.testing.assert_allclose(y64, ref, rtol=1e-12, atol=1e-12 * scale)


def test_full_size_refined_solve_vs_oracle_residual(eng):
    grid = (192, 96, 96)
    f, fixed = bcs.LOAD_CASES["edge_line"](*grid)
    x = np.random.default_rng(7).uniform(0.05, 1.0, n_elem(grid)).astype(np.float32)
    law = L.make_law("modified", 3.0)
    u = torch.zeros(n_dof(grid), dtype=torch.float64, device="cuda")
    xd = _cuda(x)
    st = eng.solve(grid, law, xd, _cuda(f), _cuda(bcs.node_mask(*grid, fixed)), u, rtol=1e-8)
    assert st["status"] == L.GBS_OK and st["relres"] <= 1e-8, st
    ug = u.cpu().numpy()
    dm = bcs.dof_mask(*grid, fixed)
    assert not ug[dm.astype(bool)].any()  # fixed DOFs stay at zero
    E = O.moduli(x.astype(np.float64), O.Material("modified", 3.0, emin=1e-9))
    fd = np.where(dm.astype(bool), 0.0, f)
    r = fd - O.apply(grid, O.ke_quadrature(), E, ug, dm)
    assert np.linalg.norm(r) <= 1.5e-8 * np.linalg.norm(fd)
    energy = torch.zeros((), dtype=torch.float64, device="cuda")
    eng.sensitivity(grid, law, xd, u, energy=energy)
    c = float(f @ ug)
    assert c > 0 and float(energy.item()) == pytest.approx(c, rel=1e-5)
