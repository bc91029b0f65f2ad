"""The evaluator row on the GPU: gbsimp_voxel_prep against the reference fixtures and the
oracle, and VoxelFEMEvaluator.evaluate / evaluate_batch against an FP64 oracle evaluation of
the same decoded grids (oracle/voxel_oracle.py + the oracle's FP64 PCG)."""
import os
import sys

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from oracle import voxel_oracle as V  # noqa: E402

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_golden import VOXEL_CASES, voxel_input  # noqa: E402


@pytest.fixture(scope="module")
def eng():
    from genpipeline_gb300.engine import get_engine

    return get_engine()


@pytest.mark.parametrize("case", VOXEL_CASES, ids=[c[0] for c in VOXEL_CASES])
def test_voxel_prep_matches_reference_fixture(eng, golden, case):
    name, shape, seed, _ = case
    ref = golden("voxel")[f"{name}_out"]
    v = torch.as_tensor(voxel_input(shape, seed), device="cuda")
    out = eng.voxel_prep(v, ref.shape).cpu().numpy()
    assert out.shape == ref.shape
    assert np.abs(out - ref).max() < 2e-6  # FP32 storage between passes on both sides
    assert np.abs(out - V.voxel_prep(voxel_input(shape, seed), ref.shape)).max() < 1e-6


def test_voxel_prep_batch_equals_single(eng):
    rng = np.random.Generator(np.random.PCG64(5))
    vols = rng.random((5, 24, 20, 18), dtype=np.float32)
    t = torch.as_tensor(vols, device="cuda")
    batch = eng.voxel_prep(t, (12, 10, 9)).cpu().numpy()
    for b in range(5):
        one = eng.voxel_prep(t[b].contiguous(), (12, 10, 9)).cpu().numpy()
        assert np.array_equal(batch[b], one)
        assert np.abs(one - V.voxel_prep(vols[b], (12, 10, 9))).max() < 1e-6


def test_smooth_voxels_numpy_roundtrip(golden):
    from genpipeline_gb300.pipeline_utils import smooth_voxels

    name, shape, seed, _ = [c for c in VOXEL_CASES if c[0] == "s_only"][0]
    out = smooth_voxels(voxel_input(shape, seed))
    assert isinstance(out, np.ndarray)
    assert np.abs(out - golden("voxel")["s_only_out"]).max() < 2e-6


def test_voxel_prep_rejects_bad_extents(eng):
    from genpipeline_gb300 import _lib as L

    v = torch.zeros((4, 4, 4), device="cuda")
    with pytest.raises(ValueError):
        eng.voxel_prep(v, (0, 4, 4))
    lib = L.load()
    assert lib.gbsimp_voxel_prep_ws_bytes(1, 4, 4, 4, 2000, 4, 4) == 0
    # a zoom of 64 -> 2 with sigma 4 needs more than 32 taps per row
    big = torch.zeros((1, 64, 8, 8), device="cuda")
    with pytest.raises(RuntimeError):
        eng.voxel_prep(big, (2, 8, 8), sigma=4.0)


def _oracle_eval(vox64: np.ndarray, force_n=1000.0):
    from genpipeline_gb300 import bcs as B

    grid = V.out_shape(vox64.shape, 0.5)
    g = V.voxel_prep(vox64, grid)
    f, fixed = B.reference_gpu(*grid, {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2}, force_n)
    E = np.maximum(g.reshape(-1), 1e-3)
    u, _, rel = O.pcg(grid, O.ke_quadrature(), E, f, B.dof_mask(*grid, fixed), tol=1e-12)
    assert rel < 1e-11
    return g, V.fem_proxies(g, u, f)


def _close(gpu, ora, g):
    n_solid = int((g > 0.5).sum())
    # one voxel within FP32 rounding of the 0.5 threshold may land on the other side
    assert abs(gpu["mass"] - ora["mass"]) <= 1.01 * 7900 / 1e9
    assert abs(gpu["compliance"] - ora["compliance"]) <= 1e-6 * abs(ora["compliance"])
    assert abs(gpu["stress"] - ora["stress_max"]) <= (1e-6 + 1.0 / n_solid) * abs(ora["stress_max"])


@pytest.fixture(scope="module")
def decoder():
    from genpipeline_gb300.designs import LatentFieldDecoder

    return LatentFieldDecoder(latent_dim=8, size=64, seed=11)


def test_evaluate_matches_oracle(eng, decoder):
    from genpipeline_gb300.fem.voxel_fem import VoxelFEMEvaluator

    ev = VoxelFEMEvaluator(use_gpu=True, engine=eng)
    z = np.random.Generator(np.random.PCG64(3)).standard_normal(8)
    res = ev.evaluate(z, decoder)
    vox = decoder.decode(torch.as_tensor(z)).cpu().numpy().reshape(64, 64, 64)
    g, ora = _oracle_eval(vox)
    assert 50 <= int((g > 0.5).sum())  # a real design, not the sentinel
    _close(res, ora, g)
    assert set(res) == {"stress", "compliance", "mass"}


def test_evaluate_batch_alone_and_in_the_mix(eng, decoder):
    from genpipeline_gb300.fem.voxel_fem import VoxelFEMEvaluator
    from genpipeline_gb300.schema import DesignParameters, FEMResult

    rng = np.random.Generator(np.random.PCG64(8))
    zs = [rng.standard_normal(8) for _ in range(5)]
    params = [DesignParameters(h_mm=10.0, r_mm=2.0, latent_z=list(z)) for z in zs]
    params.insert(2, DesignParameters(h_mm=10.0, r_mm=2.0))  # no latent: sentinel
    ev = VoxelFEMEvaluator(use_gpu=True, vae_model=decoder, engine=eng)
    out = ev.evaluate_batch(params)
    assert len(out) == 6 and all(isinstance(r, FEMResult) for r in out)
    assert out[2].success is False and out[2].stress_max == 1e6 and out[2].compliance == 1e6
    assert len(ev.evaluation_history) == 5
    alone = VoxelFEMEvaluator(use_gpu=True, engine=eng)
    for r, z in zip([o for i, o in enumerate(out) if i != 2], zs):
        one = alone.evaluate(z, decoder)
        assert r.success is True
        assert abs(r.compliance - one["compliance"]) <= 1e-7 * abs(one["compliance"])
        assert abs(r.stress_max - one["stress"]) <= 1e-7 * abs(one["stress"]) + 1e-12
        assert r.mass == one["mass"]


def test_evaluate_without_gpu_is_the_no_ccx_sentinel(decoder):
    from genpipeline_gb300.fem.voxel_fem import VoxelFEMEvaluator

    r = VoxelFEMEvaluator(use_gpu=False).evaluate(np.zeros(8), decoder)
    assert r == {"stress": 1e6, "compliance": 1e6, "mass": 1.0, "failure_reason": "no_ccx"}
