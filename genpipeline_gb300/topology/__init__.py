"""Drop-in replacements of genpipeline/topology's SIMP solvers, running on the GB300 library."""
from .simp_solver import SIMPSolver  # noqa: F401
from .simp_solver_gpu import SIMPSolverGPU  # noqa: F401
from .simp_solver_dense_gpu import DenseGPUSolver  # noqa: F401
