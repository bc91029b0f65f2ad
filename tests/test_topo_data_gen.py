"""The data generator's draws (CPU): geometry table, weights and the per-sample draw order of
topology/topo_data_gen.py:41-126,168-245 with numpy's global generator."""
import numpy as np

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
