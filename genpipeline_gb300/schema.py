"""Result records of the evaluator with the fields and defaults of genpipeline/schema.py
(``DesignParameters`` :5-14, ``FEMResult`` :16-25, ``OptimizationSample`` :27-34), as plain
dataclasses (attribute access and ``model_dump()`` as in the reference)."""
from __future__ import annotations

from dataclasses import asdict, dataclass, field
from typing import Any, Dict, List, Optional


@dataclass
class DesignParameters:
    h_mm: float
    r_mm: float
    geometry_type: str = "cantilever"
    material_name: str = "Plastic_ABS"
    material_cfg: Optional[Dict[str, Any]] = None
    latent_z: Optional[List[float]] = None

    def model_dump(self) -> dict:
        return asdict(self)


@dataclass
class FEMResult:
    stress_max: float
    compliance: float
    mass: float
    stress_mean: Optional[float] = None
    bbox: Optional[Dict[str, float]] = None
    success: bool = True

    def model_dump(self) -> dict:
        return asdict(self)


@dataclass
class OptimizationSample:
    parameters: Any
    result: FEMResult
    latent_z: Optional[List[float]] = None
    timestamp: Optional[float] = None

    def model_dump(self) -> dict:
        p = self.parameters.model_dump() if hasattr(self.parameters, "model_dump") else self.parameters
        return {"parameters": p, "result": self.result.model_dump(), "latent_z": self.latent_z,
                "timestamp": self.timestamp}
