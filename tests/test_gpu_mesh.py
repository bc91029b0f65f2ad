"""STL export row on the GPU: gbsimp_marching_cubes against the marching-cubes restatement
(oracle/mc_oracle.py; same triangles in the same order) and density_to_stl's contract
(topology/mesh_export.py:7-67)."""
import numpy as np
import pytest
import torch

from oracle import mc_oracle as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from genpipeline_gb300.engine import get_engine

    return get_engine()


def _sphere(n, c, r, k):
    x, y, z = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    d = np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2)
    return (1.0 / (1.0 + np.exp((d - r) * k))).astype(np.float32)


def _random(n, seed):
    v = np.random.Generator(np.random.PCG64(seed)).random((n, n + 3, n - 2), dtype=np.float32)
    return v


@pytest.mark.parametrize("vol,level,spacing", [
    (_sphere(36, (19.7, 20.2, 19.4), 12.31, 2.0), 0.5, (1.0, 1.0, 1.0)),
    (_random(13, 3), 0.5, (3.125, 2.5, 2.5)),
    (_random(10, 4), 0.3, (1.0, 2.0, 0.5)),
])
def test_marching_cubes_matches_oracle(eng, vol, level, spacing):
    gpu = eng.marching_cubes(torch.as_tensor(vol, device="cuda"), level, spacing).cpu().numpy()
    ref = M.marching_cubes(vol, level, spacing)
    assert gpu.shape == ref.shape
    scale = max(spacing) * max(vol.shape)
    assert np.abs(gpu - ref).max() < 2e-6 * scale


def test_triangle_count_on_a_large_grid(eng):
    v = _random(96, 7)
    n = np.zeros(256, dtype=np.int64)
    for cs in range(256):
        n[cs] = M.n_triangles(cs)
    cs = np.zeros(tuple(s - 1 for s in v.shape), dtype=np.int64)
    for q, (cx, cy, cz) in enumerate(M.CORNER):
        c = v[cx:cx + v.shape[0] - 1, cy:cy + v.shape[1] - 1, cz:cz + v.shape[2] - 1]
        cs |= (c >= np.float32(0.5)).astype(np.int64) << q
    tri = eng.marching_cubes(torch.as_tensor(v, device="cuda"), 0.5)
    assert tri.shape[0] == int(n[cs].sum())


def test_density_to_stl_contract(eng, tmp_path):
    from genpipeline_gb300.topology.mesh_export import density_to_stl, read_stl

    vol = _sphere(20, (9.6, 10.2, 9.9), 6.2, 3.0)
    p = str(tmp_path / "a.stl")
    assert density_to_stl(vol, p, threshold=0.5, voxel_size_mm=(2.0, 1.0, 1.0)) == p
    tris = read_stl(p)
    ref = M.marching_cubes(vol, 0.5, (2.0, 1.0, 1.0))
    assert tris.shape == ref.shape and np.abs(tris - ref).max() < 1e-4
    assert M.open_edges(tris.astype(np.float64), 4) == 0
    # empty design
    assert density_to_stl(np.zeros((8, 8, 8)), str(tmp_path / "e.stl")) is None
    # a level above the range moves inside it (max - 10% of the range)
    dens = (0.2 * vol).astype(np.float32)
    q = str(tmp_path / "b.stl")
    density_to_stl(dens, q, threshold=0.9)
    lvl = max(float(dens.max()) - 0.1 * (float(dens.max()) - float(dens.min())), 0.1)
    assert read_stl(q).shape == M.marching_cubes(dens, lvl).shape
    # a solid block has no surface at its own value
    with pytest.raises(ValueError):
        density_to_stl(np.ones((6, 6, 6), dtype=np.float32), str(tmp_path / "c.stl"))
