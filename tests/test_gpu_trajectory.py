"""Whole SIMP trajectories on the GPU against the FP64 oracle.

Fixtures (``tests/golden/traj_*.npz``, written by ``tests/golden/make_trajectories.py``):
the oracle's loop of ``SIMPSolver.run`` (genpipeline/topology/simp_solver.py:56-79) on the
benchmark setups, and beside it a drift study: the same loop with float32 storage of dc,
filtered dc, x and xPhys and solves stopped at rtol 1e-8. Measured drift of that study
(FP32 storage alone, no kernel involved):

    setup                         max rel. compliance   max |dxPhys|   bisection steps
    32x16x16, 50 it., modified    1.2e-7                1.2e-6         identical
    32x16x16, 50 it., reference   1.2e-7                1.4e-6         identical
    64^3, 100 it., modified       3.8e-8                1.2e-7         identical

The GPU path adds FP32 rounding of its own arithmetic (filter sums, OC update) on top of
that. Measured on a GB300: 1.4e-7 / 1.4e-6 (32x16x16 modified), 1.2e-7 / 1.1e-6 (32x16x16
reference law) and 3.8e-8 / 4.5e-7 (64^3), with identical bisection step counts: the drift
floor itself. The bounds below are the target's 1e-6 on compliance and 1e-5 on any density.

``SIMPSolverGPU.run`` and ``BatchSIMP`` are compared with ``oracle.simp_gpu_run``, the
restatement of genpipeline/topology/simp_solver_gpu.py:71-136 (its tolerance schedule, the
direct solve below 50,000 DOFs, the GPU OC variant, the compliance re-solve and the early
stop), so neither is checked only against the other.
"""
import numpy as np
import pytest
import torch

from genpipeline_gb300 import _lib as L
from genpipeline_gb300 import bcs
from genpipeline_gb300.simp import SimpProblem, SolveSpec
from oracle import oracle as O

pytestmark = pytest.mark.gpu

LAWS = {"c0": "modified", "c1": "modified", "c0ref": "ref"}

# Bounds of the benchmark trajectories (relative compliance at every iteration, largest and
# mean density difference after the last iteration).
C_REL = 1e-6
DX_MAX = {"c0": 1e-5, "c0ref": 1e-5, "c1": 1e-5}
DX_MEAN = 1e-7


def _setup(name, g):
    grid = tuple(int(v) for v in g["grid"])
    if name == "c0ref":
        f, fixed = bcs.reference_cpu(*grid, None, 1.0)
    elif name == "c0":
        f, fixed = bcs.cantilever_tip(*grid)
    else:
        f, fixed = bcs.top_patch(*grid)
    spec = SolveSpec(grid=grid, penal=3.0, rmin=float(g["rmin"]), volfrac=float(g["volfrac"]), law=LAWS[name])
    return grid, f, fixed, spec


def run_steps(name, g):
    """One ``SimpProblem.step`` per OC iteration: the path the benchmark times."""
    grid, f, fixed, spec = _setup(name, g)
    prob = SimpProblem(spec, f, fixed)
    comp, steps = [], []
    for _ in range(int(g["iters"])):
        st = prob.step()
        assert st["status"] == L.GBS_OK and st["relres"] <= 1e-8, st
        comp.append(prob.compliance())
        steps.append(prob.eng.oc_result(prob._oc_key)[1])
    final = prob.final_compliance()
    return dict(compliance=np.array(comp), steps=np.array(steps), xphys=prob.xphys.cpu().numpy(), final=final)


def run_native(name, g):
    """The whole loop in one ``gbsimp_simp_run`` call; its objective per iteration is
    sum_e E_e ce_e = u.K.u, equal to f.u at the solve's 1e-8 residual."""
    grid, f, fixed, spec = _setup(name, g)
    prob = SimpProblem(spec, f, fixed)
    xphys, obj, st = prob.eng.simp_run(grid, prob.law, prob.f, prob.mask, prob.x, prob.u, spec.volfrac,
                                       spec.rmin, int(g["iters"]), oc_variant=spec.oc_variant)
    assert st["status"] == L.GBS_OK, st
    return dict(compliance=np.array(obj), steps=None, xphys=xphys.cpu().numpy(), final=None)


def deviations(run, g):
    c = np.asarray(g["compliance"])
    rel = np.abs(run["compliance"] - c) / np.abs(c)
    dx = np.abs(run["xphys"].astype(np.float64) - g["xphys"].astype(np.float64))
    out = dict(max_rel_c=float(rel.max()), worst_iter=int(rel.argmax()), max_dx=float(dx.max()),
               mean_dx=float(dx.mean()))
    if run["final"] is not None:
        out["final_rel_c"] = abs(run["final"] - float(g["final_compliance"])) / float(g["final_compliance"])
    if run["steps"] is not None:
        out["steps_differ"] = int(np.sum(run["steps"] != g["bisect_steps"]))
    return out


@pytest.mark.parametrize("name", ["c0", "c0ref", "c1"])
def test_benchmark_trajectory_vs_oracle(golden, name):
    """32x16x16 for 50 OC iterations (modified law with the point load at (32, 8, 0), and
    SIMPSolver's own law and loads) and 64^3 with the top-patch traction for 100: compliance
    at every iteration, the closing compliance, the bisection step counts and the final
    density field against the FP64 oracle."""
    g = golden("traj_" + name)
    d = deviations(run_steps(name, g), g)
    assert d["max_rel_c"] <= C_REL, d
    assert d["final_rel_c"] <= C_REL, d
    assert d["steps_differ"] == 0, d
    assert d["max_dx"] <= DX_MAX[name] and d["mean_dx"] <= DX_MEAN, d


@pytest.mark.parametrize("name", ["c0", "c1"])
def test_native_simp_loop_vs_oracle(golden, name):
    """gbsimp_simp_run (the loop inside the library) on the same fixtures."""
    g = golden("traj_" + name)
    d = deviations(run_native(name, g), g)
    assert d["max_rel_c"] <= C_REL, d
    assert d["max_dx"] <= DX_MAX[name] and d["mean_dx"] <= DX_MEAN, d


# ---- SIMPSolverGPU.run and BatchSIMP against oracle.simp_gpu_run ---------------------------
GPU_CASES = [((20, 8, 8), 0.3, 800.0, {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2}),
             ((17, 10, 12), 0.25, 1500.0, {"fixed_face": ["x_min", "y_min"], "load_face": "x_max", "load_dof": 2,
                                           "multi_load": True, "load_pattern": "grid"}),
             ((24, 9, 7), 0.2, 300.0, {"fixed_face": "z_min", "load_face": "x_max", "load_dof": 2,
                                       "multi_load": True, "load_positions": ["top", "mid_y", "mid_z"]})]


def _oracle_gpu_run(grid, vf, force, b, n_iters, penal=3.0, rmin=1.5, **kw):
    f, fixed = bcs.reference_gpu(*grid, b, force)
    return O.simp_gpu_run(grid, rmin, penal, f, bcs.dof_mask(*grid, fixed), vf, n_iters, **kw)


def _bounds(ref, grid, vf, force, b, n_iters, **kw):
    """(compliance, density) bounds: the target's 1e-6 and 2e-5, or four times the drift of the
    oracle's own runs with float32 storage where that is larger. Some trajectories amplify
    round-off, and how much depends on where the first rounding falls: at 20x8x8 with penal
    3.5, float32 storage moves the compliance by 9e-7 after 8 iterations when the initial
    design is rounded too and by 7.7e-6 when it is not (3e-7 with penal 3); the GPU run
    measured 8.6e-6. The larger of the two variants sets the bound."""
    c_tol, x_tol = 1e-6, 2e-5
    for variant in (True, "keep_start"):
        d = _oracle_gpu_run(grid, vf, force, b, n_iters, fp32_storage=variant, **kw)
        n = min(len(d["history"]), len(ref["history"]))
        rel = np.abs(d["history"][:n] - ref["history"][:n]) / np.abs(ref["history"][:n])
        c_tol = max(c_tol, 4 * float(rel.max()))
        x_tol = max(x_tol, 4 * float(np.abs(d["xphys"] - ref["xphys"]).max()))
    return c_tol, x_tol


def gpu_run_deviation(s, xp, ref):
    hist = np.asarray(s.history)
    rel = np.abs(hist - ref["history"]) / np.abs(ref["history"])
    return dict(iterations=(len(hist), ref["iterations"]), max_rel_c=float(rel.max()),
                last_rel_c=abs(s.last_compliance - ref["last_compliance"]) / abs(ref["last_compliance"]),
                max_dx=float(np.abs(xp.ravel() - ref["xphys"]).max()))


def test_simp_solver_gpu_run_vs_oracle():
    """SIMPSolverGPU.run as the reference's callers use it (its own schedule, 12 iterations)
    against the oracle's restatement of the same loop. These grids have fewer than 50,000
    DOFs, where the reference solves directly, so every solve is exact on both sides."""
    from genpipeline_gb300.topology import SIMPSolverGPU

    for g, vf, force, b in GPU_CASES:
        s = SIMPSolverGPU(*g, penal=3.0, rmin=1.5, boundary_conditions=dict(b))
        xp = s.run(volfrac=vf, n_iters=12, force_mag=force)
        ref = _oracle_gpu_run(g, vf, force, b, 12)
        d = gpu_run_deviation(s, xp, ref)
        c_tol, x_tol = _bounds(ref, g, vf, force, b, 12)
        assert d["iterations"][0] == d["iterations"][1], (g, d)
        assert d["max_rel_c"] <= c_tol and d["last_rel_c"] <= c_tol and d["max_dx"] <= x_tol, (g, d, c_tol, x_tol)


def test_simp_solver_gpu_x_init_and_preserved_vs_oracle():
    """x_init rescaled to the volume fraction and clamped, preserved elements held at 1."""
    from genpipeline_gb300.topology import SIMPSolverGPU

    g = (12, 6, 6)
    pres = np.zeros(g, dtype=bool)
    pres[-2:, :, :2] = True
    x0 = np.random.default_rng(3).uniform(0, 1, g)
    s = SIMPSolverGPU(*g, preserved_mask=pres)
    xp = s.run(volfrac=0.4, n_iters=6, x_init=x0)
    assert np.all(xp[pres] == 1.0)
    ref = _oracle_gpu_run(g, 0.4, 1.0, None, 6, preserved=pres, x_init=x0)
    d = gpu_run_deviation(s, xp, ref)
    c_tol, x_tol = _bounds(ref, g, 0.4, 1.0, None, 6, preserved=pres, x_init=x0)
    assert d["iterations"][0] == d["iterations"][1], d
    assert d["max_rel_c"] <= c_tol and d["max_dx"] <= x_tol, (d, c_tol, x_tol)


def test_simp_solver_gpu_schedule_above_direct_limit_vs_oracle():
    """40x20x20 (54,243 DOFs): above the reference's direct-solve limit, so the schedule's
    loose tolerances (1e-4, 1e-5, 1e-6) decide the solves on both sides. Two PCGs stopped at
    the same relative residual give different displacements, so the bound is set by the
    loosest solve, not by round-off: measured 1.7e-5 on compliance and 5.3e-5 on densities,
    bounded at 1e-4 and 5e-4."""
    from genpipeline_gb300.topology import SIMPSolverGPU

    g, vf, force, b = (40, 20, 20), 0.3, 1.0, None
    s = SIMPSolverGPU(*g, penal=3.0, rmin=1.5)
    xp = s.run(volfrac=vf, n_iters=10, force_mag=force)
    ref = _oracle_gpu_run(g, vf, force, b, 10)
    d = gpu_run_deviation(s, xp, ref)
    assert d["iterations"][0] == d["iterations"][1], d
    assert d["max_rel_c"] <= 1e-4 and d["max_dx"] <= 5e-4, d


def test_batch_simp_vs_oracle():
    """BatchSIMP (all problems' solves in batched rounds) against the oracle directly."""
    from genpipeline_gb300.topology.batch_simp import BatchSIMP, SimpCase

    cases = [SimpCase(g, vf, f, dict(b), 3.5, 1.5, tag=k) for k, (g, vf, f, b) in enumerate(GPU_CASES)]
    BatchSIMP(cases).run(8)
    for c, (g, vf, force, b) in zip(cases, GPU_CASES):
        ref = _oracle_gpu_run(g, vf, force, b, 8, penal=3.5)
        c_tol, x_tol = _bounds(ref, g, vf, force, b, 8, penal=3.5)
        assert c.iterations == ref["iterations"], (g, c.iterations, ref["iterations"])
        rel = np.abs(np.asarray(c.history) - ref["history"]) / np.abs(ref["history"])
        assert rel.max() <= c_tol, (g, rel.max(), c_tol)
        assert np.abs(c.density.ravel() - ref["xphys"]).max() <= x_tol, (g, x_tol)
