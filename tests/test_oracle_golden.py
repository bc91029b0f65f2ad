"""Pins the FP64 oracle to the reference's own outputs (tests/golden/*.npz, made by
tests/golden/make_golden.py from genpipeline/topology/simp_solver.py)."""
import json
import os

import numpy as np
import pytest

from genpipeline_gb300 import bcs
from oracle import oracle as O

REF = O.Material("ref", penal=3.0)


def test_quadrature_ke(golden):
    ke = O.ke_quadrature(0.3)
    np.testing.assert_allclose(ke, golden("ke")["ke_quadrature"], rtol=0, atol=1e-15)
    assert np.abs(ke - ke.T).max() == 0.0
    w = np.linalg.eigvalsh(ke)
    assert np.sum(np.abs(w) < 1e-12) == 6 and w[6] > 0.064  # 6 rigid-body modes
    for c in range(3):
        t = np.zeros(24)
        t[c::3] = 1.0
        assert np.abs(ke @ t).max() < 1e-15


def test_reference_ke_is_not_spd(golden):
    """The reference's literal table (simp_solver.py:284-1543) is non-symmetric and
    indefinite -- the reason the solve uses the quadrature stiffness."""
    k = golden("ke")["ke_reference"]
    assert np.abs(k - k.T).max() > 0.05
    assert np.linalg.eigvalsh(0.5 * (k + k.T)).min() < -0.5


def test_edof_convention(golden):
    edof = golden("kernels")["edof_5x4x3"]
    nx, ny, nz = 5, 4, 3
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    for e in range(nx * ny * nz):
        i, j, k = e // (ny * nz), (e // nz) % ny, e % nz
        for a, (cx, cy, cz) in enumerate(corners):
            n = bcs.node_id(i + cx, j + cy, k + cz, ny, nz)
            np.testing.assert_array_equal(edof[e, 3 * a:3 * a + 3], 3 * n + np.arange(3))


@pytest.mark.parametrize("rmin", [1.5, 2.0, 3.0])
def test_filter(golden, rmin):
    g = golden("kernels")
    t = f"filter_r{rmin}"
    grid = (7, 6, 5)
    hs = O.filter_hs(grid, rmin)
    np.testing.assert_allclose(hs, g[t + "_Hs"], rtol=1e-14)
    np.testing.assert_allclose(O.density_filter(grid, rmin, g[t + "_v"], hs), g[t + "_fwd"], rtol=1e-13)
    np.testing.assert_allclose(O.density_filter(grid, rmin, g[t + "_v"], hs, transpose=True), g[t + "_adj"],
                               rtol=1e-13)


@pytest.mark.parametrize("gname,grid", [("g543", (5, 4, 3)), ("g364", (3, 6, 4))])
@pytest.mark.parametrize("kname", ["lit", "spd"])
def test_apply(golden, gname, grid, kname):
    """SIMPSolver's COO assembly (iK = kron(edof, ones((24,1))), jK = kron(edof, ones((1,24))),
    sK = Ke.ravel(); simp_solver.py:200-205, 280-281) puts Ke[r,c] at (edof[c], edof[r]): the
    assembled K is sum_e P_e^T Ke^T P_e. SIMPSolverGPU (simp_solver_gpu.py:68-69,313-326) and
    fused_spmv use Ke itself. The two agree for a symmetric Ke; for the reference's
    non-symmetric table the CPU golden is matched with Ke^T."""
    g = golden("kernels")
    ke = golden("ke")["ke_reference" if kname == "lit" else "ke_quadrature"].T
    E = O.moduli(g[f"apply_{gname}_x"], REF)
    y = O.apply(grid, ke, E, g[f"apply_{gname}_p"])
    ref = g[f"apply_{gname}_{kname}_y"]
    np.testing.assert_allclose(y, ref, rtol=1e-12, atol=1e-13 * np.abs(ref).max())


@pytest.mark.parametrize("kname", ["lit", "spd"])
def test_sensitivity_and_filter_chain(golden, kname):
    g = golden("kernels")
    ke = golden("ke")["ke_reference" if kname == "lit" else "ke_quadrature"]
    grid = (6, 3, 3)
    x = g["sens_x"]
    u = g[f"sens_{kname}_u"]
    ce, dc, _ = O.element_energy(grid, ke, x, u, REF)
    np.testing.assert_allclose(dc, g[f"sens_{kname}_dc"], rtol=1e-11, atol=1e-14 * np.abs(dc).max())
    dcf = O.density_filter(grid, 1.5, dc, transpose=True)
    np.testing.assert_allclose(dcf, g[f"sens_{kname}_dcf"], rtol=1e-11, atol=1e-14 * np.abs(dcf).max())


def test_pcg_matches_reference_direct_solve(golden):
    """FP64 Jacobi-PCG on the free DOFs == the reference's spsolve (simp_solver.py:207-213)."""
    g = golden("kernels")
    ke = golden("ke")["ke_quadrature"]
    grid = (6, 3, 3)
    f, fixed = bcs.reference_cpu(*grid, None, 1.0)
    E = O.moduli(g["sens_x"], REF)
    u, it, rel = O.pcg(grid, ke, E, f, bcs.dof_mask(*grid, fixed), tol=1e-13)
    assert rel < 1e-13 and it > 0
    ref = g["sens_spd_u"]
    np.testing.assert_allclose(u, ref, rtol=0, atol=1e-10 * np.abs(ref).max())


@pytest.mark.parametrize("rmin", [1.5, 2.0])
@pytest.mark.parametrize("vf", [0.3, 0.5])
@pytest.mark.parametrize("pres", [False, True])
def test_oc_cpu_variant(golden, rmin, vf, pres):
    g = golden("kernels")
    grid = (6, 5, 4)
    p = g["oc_pres"] if pres else None
    xn, xp, _ = O.oc(grid, rmin, g["oc_x"], g["oc_dc"], vf, preserved=p)
    tag = ("ocp" if pres else "oc") + f"_r{rmin}_v{vf}"
    np.testing.assert_allclose(xn, g[tag + "_x"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(xp, g[tag + "_xphys"], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("rmin", [1.5, 2.0])
def test_oc_gpu_variant(golden, rmin):
    g = golden("kernels")
    if f"ocgpu_r{rmin}_x" not in g.files:
        pytest.skip("no SIMPSolverGPU fixture")
    # SIMPSolverGPU._build_filter stores its weights as float32 (simp_solver_gpu.py:915),
    # so its xPhys carries ~1e-8 relative rounding against the FP64 weights here.
    xn, xp, _ = O.oc((6, 5, 4), rmin, g["oc_x"], g["oc_dc"], 0.3, variant=O.OC_GPU)
    np.testing.assert_allclose(xn, g[f"ocgpu_r{rmin}_x"], rtol=1e-7, atol=1e-12)
    np.testing.assert_allclose(xp, g[f"ocgpu_r{rmin}_xphys"], rtol=1e-7, atol=1e-12)


def test_simp_small_runs(golden):
    """Whole SIMPSolver.run trajectories (SPD stiffness injected) reproduced by the oracle."""
    g = golden("simp_small")
    ke = golden("ke")["ke_quadrature"]
    cases = json.loads(str(g["cases"]))
    for name, c in cases.items():
        grid = tuple(c["grid"])
        f, fixed = bcs.reference_cpu(*grid, c["bcs"], c["force"])
        pres = g[name + "_preserved"].astype(np.uint8) if c["preserved"] else None
        x, xp, u, comp, its = O.simp_run(grid, ke, O.Material("ref", c["penal"]), c["rmin"], f,
                                         bcs.dof_mask(*grid, fixed), c["volfrac"], c["iters"],
                                         preserved=pres, tol=1e-13)
        np.testing.assert_allclose(xp, g[name + "_xphys"], rtol=0, atol=1e-8, err_msg=name)
        assert comp == pytest.approx(float(g[name + "_compliance"]), rel=1e-9), name


@pytest.mark.slow
def test_simp_c0_reference_run(golden):
    """32x16x16, volfrac 0.3, rmin 1.5, penal 3, 50 OC iterations, reference law and BCs:
    the reference solver (SPD stiffness injected) ends at compliance 8.0604130...;
    the oracle must land within 1e-6."""
    path = os.path.join(os.path.dirname(__file__), "golden", "simp_c0.npz")
    if not os.path.exists(path):
        pytest.skip("simp_c0.npz not generated")
    g = golden("simp_c0")
    ke = golden("ke")["ke_quadrature"]
    grid = (32, 16, 16)
    f, fixed = bcs.reference_cpu(*grid, None, 1.0)
    x, xp, u, comp, its = O.simp_run(grid, ke, REF, 1.5, f, bcs.dof_mask(*grid, fixed), 0.3, 50, tol=1e-11)
    assert comp == pytest.approx(float(g["compliance"]), rel=1e-6)
    np.testing.assert_allclose(xp, g["xphys"], rtol=0, atol=1e-4)
