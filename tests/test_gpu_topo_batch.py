"""Batched SIMP (GPU): BatchSIMP against one SIMPSolverGPU per problem, and the data
generator's outputs."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tight(i):
    return 1e-10, 100000


CASES = [((20, 8, 8), 0.3, 800.0, {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2}),
         ((17, 10, 12), 0.25, 1500.0, {"fixed_face": ["x_min", "y_min"], "load_face": "x_max", "load_dof": 2,
                                       "multi_load": True, "load_pattern": "grid"}),
         ((24, 9, 7), 0.2, 300.0, {"fixed_face": "z_min", "load_face": "x_max", "load_dof": 2,
                                   "multi_load": True, "load_positions": ["top", "mid_y", "mid_z"]})]


def test_batch_simp_equals_one_solver_per_problem():
    from genpipeline_gb300.topology.batch_simp import BatchSIMP, SimpCase
    from genpipeline_gb300.topology.simp_solver_gpu import SIMPSolverGPU

    cases = [SimpCase(g, vf, f, dict(b), 3.5, 1.5, tag=k) for k, (g, vf, f, b) in enumerate(CASES)]
    BatchSIMP(cases, schedule=_tight, compliance_tol=1e-10, compliance_max_iter=100000).run(6)
    for c, (g, vf, f, b) in zip(cases, CASES):
        s = SIMPSolverGPU(nx=g[0], ny=g[1], nz=g[2], penal=3.5, rmin=1.5, boundary_conditions=dict(b))
        s.tol_schedule = _tight
        # the reference's compliance solve uses _solve's defaults; match the tight batch run
        orig = s._solve
        s._solve = lambda K, ff, fx, tol=1e-10, max_iter=100000, x0=None: orig(K, ff, fx, 1e-10, 100000, x0)
        dens = s.run(volfrac=vf, n_iters=6, force_mag=f)
        assert c.iterations == len(s.history)
        assert np.abs(c.density - dens).max() < 1e-4
        assert abs(c.last_compliance - s.last_compliance) <= 1e-6 * abs(s.last_compliance)


def test_generator_writes_samples(tmp_path):
    from genpipeline_gb300.topology.mesh_export import read_stl
    from genpipeline_gb300.topology.topo_data_gen import TopoDataGenerator

    np.random.seed(7)
    g = TopoDataGenerator(output_dir=str(tmp_path), n_iters=4, grid_size="medium", batch_size=4)
    n = g.generate(6)
    assert n == len(g.written) and n >= 5
    for rec in g.written:
        assert os.path.exists(rec["stl"]) and os.path.exists(rec["json"])
        assert len(read_stl(rec["stl"])) > 0
        with open(rec["json"]) as fh:
            r = json.load(fh)
        assert set(r) == {"stress_max", "compliance", "mass", "parameters"}
        assert r["stress_max"] == pytest.approx(0.1 * r["compliance"])
        p = r["parameters"]
        name = os.path.basename(rec["stl"])
        assert name.startswith(f"{p['geometry'][:4]}_v{int(p['volfrac'] * 100)}_f{int(p['force_n'])}_"
                               f"{p['nx']}x{p['ny']}x{p['nz']}_") and name.endswith("_mesh.stl")
        assert r["compliance"] > 0 and np.isfinite(r["compliance"])
