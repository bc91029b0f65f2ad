"""Host-side contract of VoxelFEMEvaluator (fem/voxel_fem.py:403-616 of the reference) that
needs no GPU: the CalculiX branch (use_gpu=False) returns the no_ccx sentinel, evaluate_batch
keeps one result per parameter set in order with a failed sentinel for a missing latent, the
history records OptimizationSample entries, and save_history writes them as JSON."""
import json

import numpy as np
import pytest

from genpipeline_gb300.fem.voxel_fem import VoxelFEMEvaluator
from genpipeline_gb300.pipeline_utils import FEM_SENTINEL, is_valid_fem_result
from genpipeline_gb300.schema import DesignParameters, FEMResult


class _NoDecoder:
    """Stands in for the caller's decoder; the CalculiX branch never calls it."""

    def parameters(self):
        raise AssertionError("decoder used on the CalculiX branch")


def test_calculix_branch_returns_no_ccx_sentinel():
    ev = VoxelFEMEvaluator(use_gpu=False)
    r = ev.evaluate(np.zeros(16, np.float32), _NoDecoder())
    assert r == {"stress": FEM_SENTINEL, "compliance": FEM_SENTINEL, "mass": 1.0, "failure_reason": "no_ccx"}
    assert not is_valid_fem_result(r)
    assert ev.evaluation_history == []


def test_evaluate_batch_order_sentinels_and_history(tmp_path):
    ev = VoxelFEMEvaluator(use_gpu=False, vae_model=_NoDecoder())
    params = [DesignParameters(h_mm=10.0, r_mm=2.0, latent_z=[0.1, 0.2]),
              DesignParameters(h_mm=12.0, r_mm=3.0),  # no latent: failed sentinel, no history entry
              DesignParameters(h_mm=14.0, r_mm=4.0, latent_z=np.array([0.3, 0.4]))]
    res = ev.evaluate_batch(params)
    assert len(res) == 3 and all(isinstance(r, FEMResult) for r in res)
    assert all(r.success is False and r.stress_max == FEM_SENTINEL for r in res)
    assert len(ev.evaluation_history) == 2
    assert [s.parameters.h_mm for s in ev.evaluation_history] == [10.0, 14.0]
    assert ev.evaluation_history[1].latent_z == pytest.approx([0.3, 0.4])
    path = tmp_path / "history.json"
    ev.save_history(str(path))
    data = json.loads(path.read_text())
    assert [d["parameters"]["h_mm"] for d in data] == [10.0, 14.0]
    assert data[0]["result"] == {"stress_max": FEM_SENTINEL, "compliance": FEM_SENTINEL, "mass": 1.0,
                                 "stress_mean": None, "bbox": None, "success": False}
    assert data[1]["parameters"]["latent_z"] == pytest.approx([0.3, 0.4])


def test_evaluate_batch_needs_a_decoder():
    with pytest.raises(RuntimeError):
        VoxelFEMEvaluator(use_gpu=False).evaluate_batch([DesignParameters(h_mm=1.0, r_mm=1.0, latent_z=[0.0])])
