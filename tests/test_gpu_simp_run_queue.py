"""The native SIMP loop (gbsimp_simp_run) against the Python-driven loop of the same calls,
and the native solve queue (gbsimp_queue_*) against one solve per design."""
import numpy as np
import pytest
import torch

from genpipeline_gb300 import _lib as L
from genpipeline_gb300 import bcs
from genpipeline_gb300 import designs as D
from genpipeline_gb300.batch import FEMDesign, SolveQueue, solve_plain
from genpipeline_gb300.engine import Engine, n_dof
from genpipeline_gb300.simp import SimpProblem, SolveSpec

pytestmark = pytest.mark.gpu


def test_simp_run_equals_the_python_loop():
    grid = (20, 10, 8)
    f, fixed = bcs.cantilever_tip(*grid)
    spec = SolveSpec(grid=grid, penal=3.0, rmin=1.5, volfrac=0.3, law="modified")
    prob = SimpProblem(spec, f, fixed)
    objectives = []
    for _ in range(6):
        prob.step()
        objectives.append(float(prob.energy.item()))
    eng = prob.eng
    x = torch.full((int(np.prod(grid)),), 0.3, device="cuda", dtype=torch.float32)
    u = torch.zeros(n_dof(grid), device="cuda", dtype=torch.float64)
    xphys, obj, st = eng.simp_run(grid, prob.law, prob.f, prob.mask, x, u, 0.3, 1.5, 6, oc_variant=spec.oc_variant,
                                  rtol=spec.rtol, inner_rtol=spec.inner_rtol, max_iter=spec.max_iter,
                                  max_outer=spec.max_outer)
    assert st["status"] == L.GBS_OK and len(obj) == 6
    # the same device calls in the same order: the same designs and objectives
    assert torch.equal(x, prob.x) and torch.equal(xphys, prob.xphys)
    np.testing.assert_allclose(obj, objectives, rtol=1e-12)


def test_save_state_resumes_bit_for_bit(tmp_path):
    """A run saved after four OC iterations and loaded into a fresh problem continues with
    the same designs, displacements and PCG iteration counts as the run that kept going."""
    grid = (24, 12, 10)
    f, fixed = bcs.cantilever_tip(*grid)
    spec = SolveSpec(grid=grid, penal=3.0, rmin=1.5, volfrac=0.3, law="modified")
    a = SimpProblem(spec, f, fixed)
    for _ in range(4):
        a.step()
    path = str(tmp_path / "simp_state")  # any name: the file is written under it as given
    a.save_state(path)
    b = SimpProblem(spec, f, fixed)
    b.load_state(path)
    assert b.iteration == a.iteration == 4 and b.solved == a.solved
    for _ in range(3):
        sa, sb = a.step(), b.step()
        assert sa["iterations"] == sb["iterations"] and sa["outer"] == sb["outer"]
    assert torch.equal(a.x, b.x) and torch.equal(a.xphys, b.xphys) and torch.equal(a.u, b.u)
    other = SimpProblem(SolveSpec(grid=(12, 6, 5), penal=3.0, rmin=1.5, volfrac=0.3, law="modified"),
                        *bcs.cantilever_tip(12, 6, 5))
    with pytest.raises(ValueError):
        other.load_state(path)


def test_simp_run_early_stop_rule():
    grid = (16, 8, 8)
    f, fixed = bcs.cantilever_tip(*grid)
    eng = Engine()
    law = L.make_law("modified", 3.0)
    df = torch.as_tensor(f, device="cuda")
    mask = torch.as_tensor(bcs.node_mask(*grid, fixed), device="cuda")
    x = torch.full((int(np.prod(grid)),), 0.3, device="cuda", dtype=torch.float32)
    u = torch.zeros(n_dof(grid), device="cuda", dtype=torch.float64)
    _, obj, _ = eng.simp_run(grid, law, df, mask, x, u, 0.3, 1.5, 60, early_stop=True)
    assert 4 <= len(obj) < 60
    ch = [abs(a - b) / (a + 1e-10) for a, b in zip(obj[:-1], obj[1:])]
    assert all(c < 0.01 for c in ch[-3:])  # stopped on three changes below 1%
    assert not all(c < 0.01 for c in ch[-4:-1]) or len(ch) == 3  # and not earlier


def _designs(seed0=200):
    out = []
    for k, (grid, load) in enumerate([((24, 24, 24), "cantilever"), ((16, 16, 16), "top_patch"),
                                      ((32, 16, 16), "cantilever"), ((20, 20, 20), "torsion"),
                                      ((28, 14, 14), "cantilever")]):
        if load == "cantilever":
            f, fixed = bcs.cantilever_tip(*grid)
        else:
            f, fixed = D.load_case(load, grid[0])
        out.append(FEMDesign(grid, D.grf_density(grid, seed0 + k), f, fixed, tag=k))
    return out


def test_queue_matches_one_solve_per_design():
    eng = Engine()
    plain = {d.tag: d for d in solve_plain(_designs(), eng)}
    q = SolveQueue(eng)
    designs = _designs()
    for d in designs[:3]:
        q.submit(d)
    done = q.poll()
    for d in designs[3:]:  # requests arriving while the first ones are in flight
        q.submit(d)
    for _ in range(60):
        done += q.poll(max_done=2)
        if len(q) == 0:
            break
    assert len(q) == 0 and sorted(d.tag for d in done) == list(range(5))
    for d in done:
        p = plain[d.tag]
        assert d.stats["status"] == L.GBS_OK and d.stats["relres"] <= 1e-8, d.stats
        up, uq = p.du.cpu().numpy(), d.du.cpu().numpy()
        np.testing.assert_allclose(uq, up, rtol=0, atol=1e-6 * np.abs(up).max())
        # both solves certify ||D(f - K u)|| <= 1e-8 ||D f||: f.(u1 - u2) = u.(r2 - r1) <= 2e-8 ||u|| ||D f||
        fd = np.asarray(p.f, dtype=np.float64).copy()
        fd[np.asarray(p.fixed_dofs, dtype=np.int64)] = 0.0
        assert abs(d.compliance - p.compliance) <= 4e-8 * np.linalg.norm(up) * np.linalg.norm(fd)
    q.close()
