"""Known-answer tests of the FP64 oracle's assembled operator and solver (no GPU): facts of
linear elasticity that hold for any correct hexahedral assembly, independent of the
reference's fixtures.

- Rigid motions (three translations, three infinitesimal rotations) of an unconstrained grid
  are in the null space of K(x), whatever the element moduli.
- Patch test: a uniform strain field u = G r on a homogeneous grid gives zero force at every
  interior node.
- A load case symmetric under the x and y mirrors gives a mirror-symmetric displacement.
- Compliance f.u equals the sum of the element energies sum_e E_e u_e^T Ke u_e.
"""
import numpy as np
import pytest

from genpipeline_gb300 import bcs
from oracle import oracle as O

MAT = O.Material("modified", 3.0, emin=1e-9)


def _coords(grid):
    nx, ny, nz = grid
    i, j, k = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    return np.stack([i.ravel(), j.ravel(), k.ravel()], 1).astype(np.float64)  # node order n


def _scale(grid, ke, E):
    p = np.random.default_rng(0).standard_normal(3 * int(np.prod(np.array(grid) + 1)))
    return np.abs(O.apply(grid, ke, E, p)).max()


def test_rigid_motions_are_in_the_null_space():
    grid = (7, 5, 6)
    ke = O.ke_quadrature()
    E = np.random.default_rng(1).uniform(0.01, 1.0, int(np.prod(grid)))
    r = _coords(grid) - np.array(grid) / 2.0
    scale = _scale(grid, ke, E)
    motions = [np.tile(np.eye(3)[c], (len(r), 1)) for c in range(3)]
    motions += [np.cross(np.eye(3)[a], r) for a in range(3)]  # omega x r
    for u in motions:
        assert np.abs(O.apply(grid, ke, E, u.ravel())).max() < 1e-12 * scale * np.abs(u).max()


def test_patch_test_uniform_strain():
    grid = (6, 5, 7)
    nx, ny, nz = grid
    ke = O.ke_quadrature()
    E = np.ones(int(np.prod(grid)))
    r = _coords(grid)
    g = np.random.default_rng(2).standard_normal((3, 3))
    y = O.apply(grid, ke, E, (r @ g.T).ravel()).reshape(-1, 3)
    interior = ((r[:, 0] > 0) & (r[:, 0] < nx) & (r[:, 1] > 0) & (r[:, 1] < ny) & (r[:, 2] > 0) & (r[:, 2] < nz))
    assert np.abs(y[interior]).max() < 1e-12 * np.abs(y).max()
    assert np.abs(y[~interior]).max() > 1e-3  # the boundary carries the traction


def test_symmetric_load_gives_symmetric_response():
    grid = (8, 8, 6)
    nx, ny, nz = grid
    f, fixed = bcs.LOAD_CASES["top_patch"](*grid)
    ke = O.ke_quadrature()
    x = np.random.default_rng(3).uniform(0.1, 1.0, grid)
    x = 0.25 * (x + x[::-1] + x[:, ::-1] + x[::-1, ::-1])  # densities with both mirrors
    E = O.moduli(x.ravel(), MAT)
    u, _, _ = O.pcg(grid, ke, E, f, bcs.dof_mask(*grid, fixed), tol=1e-13)
    U = u.reshape(nx + 1, ny + 1, nz + 1, 3)
    tol = 1e-9 * np.abs(U).max()
    # mirror x -> nx - x: u_x changes sign, u_y and u_z do not; likewise for y
    np.testing.assert_allclose(U[::-1, :, :, 0], -U[..., 0], atol=tol)
    np.testing.assert_allclose(U[::-1, :, :, 1:], U[..., 1:], atol=tol)
    np.testing.assert_allclose(U[:, ::-1, :, 1], -U[..., 1], atol=tol)
    np.testing.assert_allclose(U[:, ::-1, :, 0::2], U[..., 0::2], atol=tol)


@pytest.mark.parametrize("case", ["cantilever", "torsion", "edge_line"])
def test_compliance_equals_element_energy(case):
    grid = (12, 6, 8)
    f, fixed = bcs.LOAD_CASES[case](*grid)
    ke = O.ke_quadrature()
    x = np.random.default_rng(4).uniform(0.05, 1.0, int(np.prod(grid)))
    u, _, _ = O.pcg(grid, ke, O.moduli(x, MAT), f, bcs.dof_mask(*grid, fixed), tol=1e-13)
    _, _, energy = O.element_energy(grid, ke, x, u, MAT)
    assert energy == pytest.approx(float(f @ u), rel=1e-10)
