"""The data generator on CPU: geometry table, weights and the per-sample draw order of
topology/topo_data_gen.py:41-126,168-245 with numpy's global generator; the batching, the
sample records (:246-289) and the skip-on-failure rule (:301-307) with the device steps
replaced by host stand-ins."""
import numpy as np
import pytest

from genpipeline_gb300.topology.topo_data_gen import TopoDataGenerator

REF_KEYS = ["cantilever", "tapered", "ribbed", "lbracket", "bridge", "arch", "3dload", "offset", "center", "portal",
            "spoke", "tower", "sandwich", "simply", "branch", "y_tree", "network"]


def _reference_draw(gen, grid_size):
    """The draws of TopoDataGenerator.generate_single in the reference's order."""
    geoms = list(gen.GEOM_BCS.keys())
    w = np.array([gen.GEOM_WEIGHTS.get(g, 1) for g in geoms], dtype=np.float64)
    geom = np.random.choice(geoms, p=w / w.sum())
    r = np.random.randint
    if grid_size == "small":
        dims = (16, 8, 8)
    elif geom in ("lbracket", "bridge", "arch", "center"):
        dims = (r(16, 24), r(6, 10), r(12, 18))
    elif geom in ("3dload", "offset"):
        dims = (r(22, 32), r(8, 12), r(8, 12))
    elif geom in ("branch", "y_tree", "network"):
        dims = (r(22, 32), r(10, 16), r(10, 16))
    else:
        dims = (r(20, 32), r(6, 10), r(6, 10))
    return str(geom), tuple(int(v) for v in dims), np.random.uniform(0.12, 0.35), np.random.uniform(200, 5000)


def test_table_and_weights(tmp_path):
    g = TopoDataGenerator(output_dir=str(tmp_path))
    assert list(g.GEOM_BCS) == REF_KEYS
    assert g.GEOM_BCS["network"]["load_pattern"] == "grid" and g.GEOM_BCS["3dload"]["load_dof"] == [1, 2]
    assert g.GEOM_WEIGHTS["bridge"] == 2 and "portal" not in g.GEOM_WEIGHTS


def test_draw_order_matches_reference(tmp_path):
    for grid_size in ("medium", "small"):
        g = TopoDataGenerator(output_dir=str(tmp_path), grid_size=grid_size)
        np.random.seed(1234)
        ours = [g._draw() for _ in range(40)]
        np.random.seed(1234)
        ref = [_reference_draw(g, grid_size) for _ in range(40)]
        for c, (geom, dims, vf, force) in zip(ours, ref):
            assert c.tag == geom and c.grid == dims and c.volfrac == vf and c.force_mag == force
            assert c.bcs == g.GEOM_BCS[geom] and c.penal == 3.5 and c.rmin == 1.5


def _fake_pipeline(monkeypatch, g, fail_tags=()):
    """Replaces the device steps (batched SIMP, STL export) by host stand-ins; records the
    batches that reach the solver."""
    import genpipeline_gb300.topology.topo_data_gen as T

    batches = []

    def solve(cases):
        batches.append([c.grid for c in cases])
        for k, c in enumerate(cases):
            c.density = np.full(c.grid, 0.25 + 0.01 * k)
            c.last_compliance = 40.0 + k
            c.failed = c.tag in fail_tags
        return cases

    def stl(density, path, threshold=0.5, voxel_size_mm=None):
        open(path, "wb").close()
        return path

    monkeypatch.setattr(g, "_solve", solve)
    monkeypatch.setattr(T, "density_to_stl", stl)
    return batches


@pytest.mark.parametrize("method", ["generate", "generate_scaled"])
def test_generate_batches_records_and_failures(tmp_path, monkeypatch, method):
    """generate / generate_scaled split the samples into batches, consume the draws in the
    reference's order, write the reference's JSON record per sample and skip a failed
    sample (logged, not raised), returning the number written."""
    import json

    g = TopoDataGenerator(output_dir=str(tmp_path), batch_size=3)
    np.random.seed(77)
    expect = [g._draw() for _ in range(7)]
    fail = {expect[4].tag}
    batches = _fake_pipeline(monkeypatch, g, fail_tags=fail)
    np.random.seed(77)
    n = g.generate(7) if method == "generate" else g.generate_scaled(7, batch_size=3)
    assert batches == [[c.grid for c in expect[:3]], [c.grid for c in expect[3:6]], [expect[6].grid]]
    kept = [(i, c) for i, c in enumerate(expect) if c.tag not in fail]
    assert n == len(kept) == len(g.written)
    for rec, (i, c) in zip(g.written, kept):
        data = json.loads(open(rec["json"]).read())
        nx, ny, nz = c.grid
        assert data["compliance"] == 40.0 + i % 3  # the stand-in solver's value for this sample
        assert data["stress_max"] == pytest.approx(0.1 * data["compliance"], rel=1e-15)
        assert data["parameters"] == {"geometry": c.tag, "volfrac": c.volfrac, "force_n": c.force_mag,
                                      "nx": nx, "ny": ny, "nz": nz, "penal": 3.5}
        box = 100.0 * 20.0 * (100.0 if c.tag in ("lbracket", "bridge", "arch") else 20.0)
        assert data["mass"] == pytest.approx((0.25 + 0.01 * (i % 3)) * box * 1.05e-6, rel=1e-12)
        stem = f"{c.tag[:4]}_v{int(c.volfrac * 100)}_f{int(c.force_mag)}_{nx}x{ny}x{nz}_"
        assert rec["stl"].rsplit("/", 1)[1].startswith(stem) and rec["stl"].endswith("_mesh.stl")
        assert rec["json"].endswith("_fem_results.json")


def test_sensitivity_solve_schedule():
    """(tol, max_iter) of each SIMP iteration's sensitivity solve, as SIMPSolverGPU.run sets
    them (topology/simp_solver_gpu.py:94-100): 1e-4/200 for iterations 0-2, 1e-5/400 for 3-7,
    1e-6/800 after."""
    from genpipeline_gb300.topology.batch_simp import reference_schedule
    from genpipeline_gb300.topology.simp_solver_gpu import SIMPSolverGPU

    got = [reference_schedule(i) for i in (0, 2, 3, 7, 8, 79)]
    assert got == [(1e-4, 200), (1e-4, 200), (1e-5, 400), (1e-5, 400), (1e-6, 800), (1e-6, 800)]
    assert SIMPSolverGPU.tol_schedule is reference_schedule


def test_generator_bcs_cover_every_geometry(tmp_path):
    from genpipeline_gb300 import bcs as B

    g = TopoDataGenerator(output_dir=str(tmp_path))
    for geom, b in g.GEOM_BCS.items():
        nx, ny, nz = 20, 9, 11
        f, fixed = B.generator(nx, ny, nz, b, 1000.0)
        f_cpu, fixed_cpu = B.reference_cpu(nx, ny, nz, b, 1000.0)
        assert np.array_equal(np.sort(fixed), np.sort(fixed_cpu)), geom
        assert len(fixed) > 0, geom  # (unknown face names fall back as in the reference, "spoke" loads a clamped node)
        if b.get("multi_load") and (b.get("load_positions") or b.get("load_pattern") == "grid"):
            assert f.sum() < 0 and not np.array_equal(f, f_cpu), geom
        else:
            assert np.array_equal(f, f_cpu), geom
        assert np.isfinite(f).all() and np.abs(f).sum() > 0, geom
