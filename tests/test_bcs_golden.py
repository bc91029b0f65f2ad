"""Host boundary-condition logic against the reference's own _get_bcs outputs."""
import json

import numpy as np
import pytest

from genpipeline_gb300 import bcs


def _cases(golden, key):
    return json.loads(str(golden("bcs")[key]))


def test_cpu_bcs_match_reference(golden):
    g = golden("bcs")
    cases = _cases(golden, "cases")
    n = 0
    for gx, gy, gz in ((6, 4, 5), (7, 3, 4)):
        for name, spec in cases.items():
            f, fixed = bcs.reference_cpu(gx, gy, gz, spec, force_mag=2.5)
            tag = f"cpu_{gx}{gy}{gz}_{name}"
            np.testing.assert_array_equal(fixed, g[tag + "_fixed"], err_msg=tag)
            np.testing.assert_allclose(f, g[tag + "_f"], rtol=0, atol=1e-15, err_msg=tag)
            n += 1
    assert n == 2 * len(cases)


def test_gpu_bcs_match_reference(golden):
    g = golden("bcs")
    cases = _cases(golden, "gpu_cases")
    for gx, gy, gz in ((6, 4, 5), (7, 3, 8)):
        for name, spec in cases.items():
            tag = f"gpu_{gx}{gy}{gz}_{name}"
            if tag + "_f" not in g.files:
                pytest.skip("reference GPU-class fixtures were not generated")
            f, fixed = bcs.reference_gpu(gx, gy, gz, spec, force_mag=2.5)
            np.testing.assert_array_equal(fixed, g[tag + "_fixed"], err_msg=tag)
            np.testing.assert_allclose(f, g[tag + "_f"], rtol=0, atol=1e-15, err_msg=tag)


def test_node_mask_roundtrip():
    f, fixed = bcs.reference_cpu(5, 3, 4, {"fixed_face": ["x_min", "z_max"]})
    m = bcs.node_mask(5, 3, 4, fixed)
    back = np.flatnonzero(np.unpackbits(m[:, None], axis=1, bitorder="little")[:, :3].ravel())
    np.testing.assert_array_equal(back, fixed)


@pytest.mark.parametrize("case", sorted(bcs.LOAD_CASES))
def test_benchmark_load_cases(case):
    nx, ny, nz = 16, 8, 12
    f, fixed = bcs.LOAD_CASES[case](nx, ny, nz)
    assert f.shape == (3 * (nx + 1) * (ny + 1) * (nz + 1),)
    assert not np.any(f[fixed])  # no load on a clamped DOF
    F = f.reshape(-1, 3)
    if case == "torsion":
        np.testing.assert_allclose(F.sum(0), 0.0, atol=1e-12)
        jj, kk = np.meshgrid(np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
        ids = bcs.node_id(nx, jj.ravel(), kk.ravel(), ny, nz)
        torque = np.sum((jj.ravel() - ny / 2) * F[ids, 2] - (kk.ravel() - nz / 2) * F[ids, 1])
        assert torque == pytest.approx(1.0)
    else:
        np.testing.assert_allclose(F.sum(0), [0.0, 0.0, -1.0], atol=1e-12)


def test_cantilever_point_location():
    f, fixed = bcs.cantilever_tip(32, 16, 16)
    (d,) = np.flatnonzero(f)
    assert d == 3 * bcs.node_id(32, 8, 0, 16, 16) + 2 and f[d] == -1.0
    assert len(fixed) == 3 * 17 * 17


def test_solver_bc_cache_equals_a_fresh_build():
    """SIMPSolverGPU's device cache of its boundary conditions (exercised on CPU tensors):
    every call equals a fresh host build, hands out tensors of its own, and follows changes of
    the force and of the boundary-condition dictionary; the node mask follows the fixed set."""
    import torch

    from genpipeline_gb300.topology.simp_solver_gpu import _BcCache

    grid = (7, 3, 8)
    cache = _BcCache(grid, torch.device("cpu"))
    spec = {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2}
    for force, spec_now in ((2.5, spec), (2.5, spec), (1.0, spec), (1.0, dict(spec, load_dof=1)),
                            (1.0, dict(spec, fixed_face=["x_min", "z_min"])), (1.0, spec)):
        f, fixed = cache.bcs(spec_now, force)
        f_ref, fixed_ref = bcs.reference_gpu(*grid, spec_now, force)
        np.testing.assert_array_equal(f.numpy(), f_ref)
        np.testing.assert_array_equal(fixed.numpy(), fixed_ref)
        assert f.dtype == torch.float64 and fixed.dtype == torch.int64
        f.mul_(7.0)  # the caller's copy: the next call is unaffected
        np.testing.assert_array_equal(cache.mask(fixed).numpy(), bcs.node_mask(*grid, fixed_ref))
    np.testing.assert_array_equal(cache.bcs(spec, 1.0)[0].numpy(), bcs.reference_gpu(*grid, spec, 1.0)[0])
    other = np.array([0, 1, 2, 30], dtype=np.int64)
    np.testing.assert_array_equal(cache.mask(torch.as_tensor(other)).numpy(), bcs.node_mask(*grid, other))
