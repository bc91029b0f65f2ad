"""GB300-native (sm_103a) 3D SIMP / voxel-FEM hot path behind the reference's topology/
solver, fem/ GPU-evaluator and cuda_kernels signatures.

The compute is hand-written CUDA in ``libgbsimp.so`` (C ABI: ``include/gbsimp.h``); this
package is the host side. There is no CPU fallback: without the library or a GPU the
entry points raise.
"""
from . import bcs  # noqa: F401

__all__ = ["bcs"]
