"""The pieces of genpipeline/pipeline_utils.py that sit around the FEM evaluator.

``smooth_voxels`` (pipeline_utils.py:55-76) runs on the device (gbsimp_voxel_prep with no
resampling): Gaussian blur of ``sigma`` voxels with the mirror boundary, then the logistic
sharpening. It accepts a numpy array (returned as numpy, like the reference) or a CUDA
tensor (returned on the device); there is no CPU fallback. The FEM sentinel constants and
``is_valid_fem_result`` keep the reference's values and rule (:18-33).
"""
from __future__ import annotations

import json

import numpy as np
import torch

FEM_SENTINEL: float = 1e6
FEM_VALID_THRESHOLD: float = 1e5


def is_valid_fem_result(result) -> bool:
    """True when the result looks like a real FEM output (0 < stress < 1e5)."""
    from .schema import FEMResult

    if isinstance(result, FEMResult):
        stress = result.stress_max
    elif isinstance(result, dict):
        stress = result.get("stress", result.get("stress_max", FEM_SENTINEL))
    else:
        stress = FEM_SENTINEL
    return 0.0 < float(stress) < FEM_VALID_THRESHOLD


class NumpyEncoder(json.JSONEncoder):
    """JSON encoder for numpy values and result records."""

    def default(self, obj):
        if isinstance(obj, np.ndarray):
            return obj.tolist()
        if isinstance(obj, np.integer):
            return int(obj)
        if isinstance(obj, np.floating):
            return float(obj)
        if hasattr(obj, "model_dump") and callable(obj.model_dump):
            return obj.model_dump()
        return super().default(obj)


def smooth_voxels(voxels, sigma: float = 0.5, sharpness: float = 15.0):
    from .engine import get_engine

    if isinstance(voxels, torch.Tensor):
        v = voxels.to(dtype=torch.float32).contiguous()
        return get_engine(v.device).voxel_prep(v, tuple(v.shape[-3:]), sigma, sharpness)
    if not torch.cuda.is_available():
        raise RuntimeError("smooth_voxels runs on the GPU (no CPU fallback)")
    v = torch.as_tensor(np.ascontiguousarray(voxels, dtype=np.float32), device="cuda")
    return get_engine(v.device).voxel_prep(v, tuple(v.shape), sigma, sharpness).cpu().numpy()
