"""Drop-in replacement of genpipeline/fem's GPU evaluator on the GB300 library."""
from .gpu_fem_solver import GPUConjugateGradientFEM, GPUVoxelFEM  # noqa: F401
