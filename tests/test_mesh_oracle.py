"""STL export row on the CPU: the marching-cubes restatement (oracle/mc_oracle.py) on
analytic shapes, and the library's case table against the restatement (the table is built
by host code, so this runs without a GPU)."""
import ctypes as C

import numpy as np
import pytest

from oracle import mc_oracle as M


def _sphere(n, c, r, k):
    x, y, z = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    d = np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2)
    return 1.0 / (1.0 + np.exp((d - r) * k))


@pytest.mark.parametrize("r,c,k", [(12.31, (19.7, 20.2, 19.4), 2.0), (7.1, (10.5, 10.5, 10.5), 4.0)])
def test_sphere_area_volume_closed_outward(r, c, k):
    tr = M.marching_cubes(_sphere(36, c, r, k), 0.5)
    assert abs(M.area(tr) / (4 * np.pi * r ** 2) - 1) < 5e-3
    assert abs(M.enclosed_volume(tr) / (4 / 3 * np.pi * r ** 3) - 1) < 2e-2
    assert M.open_edges(tr) == 0
    n = np.cross(tr[:, 1] - tr[:, 0], tr[:, 2] - tr[:, 0])
    assert np.all(np.einsum("ij,ij->i", n, tr.mean(axis=1) - np.array(c)) > 0)


def test_random_field_is_closed():
    v = np.random.Generator(np.random.PCG64(1)).random((14, 14, 14))
    v[[0, -1], :, :] = 0
    v[:, [0, -1], :] = 0
    v[:, :, [0, -1]] = 0
    tr = M.marching_cubes(v, 0.5)
    assert len(tr) > 1000 and M.open_edges(tr, 7) == 0


def test_every_case_loops_close_on_faces():
    for cs in range(256):
        edges = [e for lp in M.TABLE[cs] for e in lp]
        cut = [e for e, (a, b) in enumerate(M.EDGE) if ((cs >> a) & 1) != ((cs >> b) & 1)]
        assert sorted(edges) == cut


def test_library_table_equals_restatement():
    from genpipeline_gb300 import _lib as L

    lib = L.load()
    ntri = (C.c_ubyte * 256)()
    nloop = (C.c_ubyte * 256)()
    ln = (C.c_ubyte * (256 * 4))()
    edge = (C.c_byte * (256 * 12))()
    mx = lib.gbsimp_marching_cubes_table(ntri, nloop, ln, edge)
    assert mx >= max(M.n_triangles(cs) for cs in range(256))
    for cs in range(256):
        loops = M.TABLE[cs]
        assert nloop[cs] == len(loops) and ntri[cs] == M.n_triangles(cs)
        e0 = 0
        for q, lp in enumerate(loops):
            assert ln[cs * 4 + q] == len(lp)
            assert [edge[cs * 12 + e0 + t] for t in range(len(lp))] == lp
            e0 += len(lp)


def test_stl_roundtrip(tmp_path):
    from genpipeline_gb300.topology.mesh_export import read_stl, write_stl

    tr = M.marching_cubes(_sphere(12, (5.5, 5.5, 5.5), 3.3, 3.0), 0.5).astype(np.float32)
    p = tmp_path / "s.stl"
    write_stl(str(p), tr)
    assert p.stat().st_size == 84 + 50 * len(tr)
    assert np.array_equal(read_stl(str(p)), tr)
