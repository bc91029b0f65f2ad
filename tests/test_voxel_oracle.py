"""The evaluator's input step and outputs (CPU): the FP64 restatement in
oracle/voxel_oracle.py against the reference's own results (tests/golden/voxel.npz, made by
tests/golden/make_golden.py from scipy.ndimage.zoom + pipeline_utils.smooth_voxels)."""
import os
import sys

import numpy as np
import pytest

from oracle import voxel_oracle as V

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_golden import VOXEL_CASES, voxel_input  # noqa: E402


@pytest.mark.parametrize("case", VOXEL_CASES, ids=[c[0] for c in VOXEL_CASES])
def test_voxel_prep_matches_reference(golden, case):
    name, shape, seed, _ = case
    ref = golden("voxel")[f"{name}_out"]
    out = V.voxel_prep(voxel_input(shape, seed), ref.shape)
    # the reference rounds to float32 after the zoom and after each filter axis
    assert np.abs(out - ref).max() < 1e-6


def test_voxel_inputs_are_the_recorded_ones(golden):
    g = golden("voxel")
    for name, shape, seed, _ in VOXEL_CASES:
        if f"{name}_in" in g.files:
            assert np.array_equal(g[f"{name}_in"], voxel_input(shape, seed))


def test_out_shape_follows_scipy_rounding():
    assert V.out_shape((64, 64, 64), 0.5) == (32, 32, 32)
    assert V.out_shape((20, 17, 9), 0.5) == (10, 8, 4)


def test_filter_rows_sum_to_one():
    for n_in, n_out in [(64, 32), (17, 8), (9, 9)]:
        a = V.gauss_matrix(n_out, 0.5) @ V.zoom_matrix(n_in, n_out)
        assert np.allclose(a.sum(axis=1), 1.0)
    assert np.allclose(V.gauss_matrix(7, 0.0), np.eye(7))


def test_scipy_agrees_on_fresh_inputs():
    nd = pytest.importorskip("scipy.ndimage")
    v = np.random.Generator(np.random.PCG64(99)).random((14, 11, 22)).astype(np.float32)
    z = nd.zoom(v, 0.5, order=1)
    g = nd.gaussian_filter(z, sigma=0.5)
    ref = 1.0 / (1.0 + np.exp(-15.0 * (g - 0.5)))
    assert np.abs(V.voxel_prep(v, z.shape) - ref).max() < 1e-6


def test_fem_proxies_sentinel_and_mass():
    vox = np.zeros((8, 8, 8))
    f = np.zeros(3 * 9 ** 3)
    u = np.zeros_like(f)
    r = V.fem_proxies(vox, u, f)
    assert r["stress_max"] == 1e4 and r["compliance"] == 1e6 and r["displacement_max"] == 1e3
    assert r["mass"] == 0.0
    vox[:] = 1.0
    f[5] = -1.0
    u[5] = -20.0
    r = V.fem_proxies(vox, u, f)
    assert r["compliance"] == 20.0 and np.isclose(r["stress_max"], 20.0 / 512 * 10.0)
    assert np.isclose(r["mass"], 512 * 7900 / 1e9)
