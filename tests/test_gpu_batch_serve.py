"""Batched solves and the serving loop: every result equals the same solve done alone."""
import numpy as np
import pytest
import torch

from genpipeline_gb300 import _lib as L
from genpipeline_gb300 import designs as D
from genpipeline_gb300.batch import BatchFEM, FEMDesign, solve_plain
from genpipeline_gb300.engine import Engine
from genpipeline_gb300.serve import FEMServer, request_stream

pytestmark = pytest.mark.gpu

# Every design is solved to ||D(f - K u)|| <= 1e-8 ||D f|| on both paths, so displacements
# agree to ~1e-6 of their maximum. Two such solutions u1, u2 have compliances that differ by
# f.(u1 - u2) = u.(r2 - r1) (K symmetric), at most 2e-8 ||u|| ||D f||: the tests allow twice that.
U_TOL, RELRES = 1e-6, 1e-8


def _c_bound(u, f, fixed):
    fd = np.asarray(f, dtype=np.float64).copy()
    fd[np.asarray(fixed, dtype=np.int64)] = 0.0
    return 4 * RELRES * float(np.linalg.norm(u)) * float(np.linalg.norm(fd))


def _designs():
    out = []
    for k, (grid, load) in enumerate([((24, 24, 24), "cantilever"), ((32, 32, 32), "top_patch"),
                                      ((40, 20, 20), "cantilever"), ((16, 16, 16), "torsion"),
                                      ((48, 24, 12), "cantilever")]):
        if load == "cantilever":
            from genpipeline_gb300 import bcs
            f, fixed = bcs.cantilever_tip(*grid)
        else:
            f, fixed = D.load_case(load, grid[0])
        out.append(FEMDesign(grid, D.grf_density(grid, 100 + k), f, fixed))
    return out


@pytest.mark.parametrize("fused,round_iters,share,group", [(True, 0, 0, 0), (False, 0, 0, 0), (True, 7, 0, 0),
                                                           (False, 30, 0, 0), (True, 0, 1, 0), (True, 13, 1, 2)])
def test_batch_equals_single_solves(fused, round_iters, share, group):
    """Whole inner solves per round, and rounds of 7 (persistent kernel) or 30 (graph loop, two
    12-iteration trips, then three) inner iterations after which each solve is paused and
    resumed in the next round; SM shares by element count or by element count x extent, and
    launches of at most two designs (a paused design then resumes under another plan)."""
    eng = Engine()
    single = solve_plain(_designs(), eng)
    bf = BatchFEM(eng, fused=fused, round_iters=round_iters)
    bf.opts.batch_share, bf.opts.batch_group = share, group
    batch = bf.solve_all(_designs())
    assert len(batch) == len(single)
    by_grid = {d.grid: d for d in batch}
    for s in single:
        b = by_grid[s.grid]
        assert b.stats["status"] == L.GBS_OK and b.stats["relres"] <= 1e-8, b.stats
        us, ub = s.du.cpu().numpy(), b.du.cpu().numpy()
        np.testing.assert_allclose(ub, us, rtol=0, atol=U_TOL * np.abs(us).max())
        assert abs(b.compliance - s.compliance) <= _c_bound(us, s.f, s.fixed_dofs)


def test_autotuned_batch_equals_single_solves(tmp_path):
    """The tuner times every candidate on copies of the designs, applies the fastest, and the
    solutions are those of single solves."""
    from genpipeline_gb300.autotune import CANDIDATES, BatchTuner, summary

    eng = Engine()
    tuner = BatchTuner(cache_path=str(tmp_path / "tune.json"))
    single = solve_plain(_designs(), eng)
    bf = BatchFEM(eng, tuner=tuner)
    batch = bf.solve_all(_designs())
    grids = [d.grid for d in batch]
    s = summary(tuner, grids)
    assert bf.config is not None and tuner.choice(grids) == bf.config
    assert len(s["trial_seconds"]) == len(CANDIDATES) and all(t > 0 for t in s["trial_seconds"].values())
    by_grid = {d.grid: d for d in batch}
    for d in single:
        b = by_grid[d.grid]
        assert b.stats["status"] == L.GBS_OK and b.stats["relres"] <= 1e-8, b.stats
        assert abs(b.compliance - d.compliance) <= _c_bound(d.du.cpu().numpy(), d.f, d.fixed_dofs)


def test_serving_results_equal_alone_and_in_the_mix():
    eng = Engine()
    reqs = request_stream(40, rate=2000.0, edges=(16, 24, 32), repeat_frac=0.15, seed=7)
    srv = FEMServer(eng, max_slots=8, keep_solutions=True)
    summary = srv.run(reqs, realtime=True)
    assert summary["requests"] == 40 and summary["failed"] == 0
    assert summary["max_active"] > 1  # requests overlapped on the device
    assert summary["warm_starts"] >= 1
    for r in reqs:
        grid = (r.n, r.n, r.n)
        f, fixed = D.load_case(r.load, r.n)
        alone = solve_plain([FEMDesign(grid, D.grf_density(grid, r.seed), f, fixed)], eng)[0]
        ua = alone.du.cpu().numpy()
        assert abs(r.compliance - alone.compliance) <= _c_bound(ua, f, fixed), r
        np.testing.assert_allclose(r.u.cpu().numpy(), ua, rtol=0, atol=U_TOL * np.abs(ua).max())
    warm = [r for r in reqs if r.warm]
    cold = {(r.n, r.seed, r.load): r.iterations for r in reqs if not r.warm}
    assert all(r.iterations <= cold[(r.n, r.seed, r.load)] for r in warm)
