"""CPU checks (FP64 numpy) of the modal element form that the FP32 apply kernel is built on.

With T = T8 (x) I3, T8[a][m] = prod_d (m_d ? s(c_d(a)) : 1), s(0) = -1, s(1) = +1 (the 2x2x2
Walsh-Hadamard basis of the corner values, corners in the reference's local node order,
topology/simp_solver.py:251-282), Ke = T Km T^T with Km = T^T Ke T / 64. For an isotropic cube
element, Km has 45 nonzeros in a pattern that does not depend on Poisson's ratio: the three
translation modes have zero rows and columns, and the other 21 indices form 11 independent
blocks of 1-3 indices holding at most 8 distinct values. The library checks an installed Ke
against that pattern and uses the dense 24x24 kernel when it does not fit.
"""
import numpy as np
import pytest
import scipy.sparse as sp
from scipy.sparse.csgraph import connected_components

from oracle import oracle as O

CORNERS = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]


def _t24():
    t8 = np.empty((8, 8))
    for a, c in enumerate(CORNERS):
        for m in range(8):
            bits = ((m >> 2) & 1, (m >> 1) & 1, m & 1)  # mode bits (x, y, z)
            t8[a, m] = np.prod([(1.0 if c[d] else -1.0) if bits[d] else 1.0 for d in range(3)])
    return np.kron(t8, np.eye(3))


def _pattern(km):
    return np.abs(km) > 1e-12 * np.abs(km).max()


def test_basis_is_orthogonal():
    t = _t24()
    np.testing.assert_array_equal(t.T @ t, 8.0 * np.eye(24))


@pytest.mark.parametrize("nu", [0.2, 0.3, 0.35, 0.45])
def test_modal_pattern(nu):
    t = _t24()
    ke = O.ke_quadrature(nu)
    km = t.T @ ke @ t / 64.0
    np.testing.assert_allclose(t @ km @ t.T, ke, rtol=0, atol=1e-14 * np.abs(ke).max())
    nz = _pattern(km)
    assert nz.sum() == 45
    np.testing.assert_array_equal(nz, _pattern(t.T @ O.ke_quadrature(0.3) @ t))  # same for every nu
    rows = np.flatnonzero(nz.any(axis=1))
    np.testing.assert_array_equal(rows, np.arange(3, 24))  # translation modes (m = 0) drop out
    n_blocks, labels = connected_components(sp.csr_matrix(nz[np.ix_(rows, rows)]), directed=False)
    sizes = np.bincount(labels)
    assert n_blocks == 11 and sizes.min() >= 1 and sizes.max() <= 3
    assert len(np.unique(np.round(km[nz] / np.abs(km).max(), 9))) <= 8


def test_modal_product_equals_dense_product():
    """q = T^T p, r = E Km q, y = T r reproduces E Ke p, and a rigid translation of p gives 0."""
    t = _t24()
    ke = O.ke_quadrature(0.3)
    km = t.T @ ke @ t / 64.0
    rng = np.random.default_rng(3)
    p = rng.standard_normal((24, 50))
    e = rng.uniform(1e-9, 1.0, 50)
    y = t @ (e * (km @ (t.T @ p)))
    np.testing.assert_allclose(y, e * (ke @ p), rtol=0, atol=1e-12 * np.abs(ke @ p).max())
    shift = np.tile(rng.standard_normal(3), 8)  # the same displacement at every corner
    assert np.abs(km @ (t.T @ shift)).max() < 1e-13


def test_perturbed_ke_leaves_the_pattern():
    """A symmetric entry outside the pattern shows in Km (that Ke goes to the dense kernel)."""
    t = _t24()
    ke = O.ke_quadrature(0.3).copy()
    ke[0, 9] += 1e-6
    ke[9, 0] += 1e-6
    assert _pattern(t.T @ ke @ t / 64.0).sum() > 45
