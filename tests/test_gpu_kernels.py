"""CUDA kernels (through the C ABI) against the FP64 oracle and the reference fixtures.

Tolerances: FP64 paths 1e-12 relative; FP32 apply 2e-6 of max|y| (FP32 products of an
element stiffness with entries <= 0.24 and up to 24 terms); sensitivities 1e-6 relative
(FP64 compute, FP32 output); filter 1e-6; OC 1e-5 (FP32 trial densities).
"""
import json

import numpy as np
import pytest
import torch

from genpipeline_gb300 import _lib as L
from genpipeline_gb300 import bcs
from genpipeline_gb300.engine import Engine, n_dof
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GRIDS = [(1, 1, 1), (3, 5, 2), (5, 4, 3), (33, 7, 5), (6, 40, 3), (17, 9, 37)]


@pytest.fixture(scope="module")
def eng():
    return Engine()


@pytest.fixture(scope="module")
def ke_lit(golden):
    return golden("ke")["ke_reference"]


def _rand(grid, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = grid
    x = rng.uniform(0.0, 1.0, nx * ny * nz).astype(np.float32)
    x[: min(3, x.size)] = [0.0, 5e-4, 1.0][: min(3, x.size)]
    p = rng.standard_normal(n_dof(grid))
    return x, p


def _cuda(a, dtype=None):
    t = torch.as_tensor(np.ascontiguousarray(a)).cuda()
    return t if dtype is None else t.to(dtype)


def _mat(law):
    return O.Material(law, penal=3.0, emin=1e-9)


@pytest.mark.parametrize("grid", GRIDS)
@pytest.mark.parametrize("law", ["ref", "modified"])
@pytest.mark.parametrize("masked", [False, True])
def test_apply_vs_oracle(eng, grid, law, masked):
    x, p = _rand(grid, hash((grid, law, masked)) % 2**32)
    ke = O.ke_quadrature()
    E = O.moduli(x.astype(np.float64), _mat(law))
    fixed = bcs.reference_cpu(*grid, {"fixed_face": ["x_min", "z_max"]})[1] if masked else None
    dm = bcs.dof_mask(*grid, fixed) if masked else None
    ref = O.apply(grid, ke, E, p, dm)
    lw = L.make_law(law, 3.0)
    m = _cuda(bcs.node_mask(*grid, fixed)) if masked else None
    y64 = eng.apply(grid, lw, _cuda(x), _cuda(p), m).cpu().numpy()
    np.testing.assert_allclose(y64, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    y32 = eng.apply(grid, lw, _cuda(x), _cuda(p, torch.float32), m).cpu().numpy()
    np.testing.assert_allclose(y32, ref, rtol=0, atol=2e-6 * np.abs(ref).max())


def _perturbed_ke():
    """SPD quadrature Ke plus a tiny symmetric term outside the modal pattern: it forces the
    dense kernel while staying numerically the same operator to ~1e-10."""
    ke = O.ke_quadrature()
    d = np.zeros((24, 24))
    d[0, 9] = d[9, 0] = 1e-10
    return ke + d


@pytest.mark.parametrize("grid", [(1, 1, 1), (33, 7, 5), (17, 9, 37), (40, 64, 64), (3, 2, 450)])
@pytest.mark.parametrize("masked", [False, True])
def test_modal_and_dense_kernels_agree(eng, grid, masked):
    nx, ny, nz = grid
    dense = Engine(ke=_perturbed_ke())
    assert dense.apply_path(nz) == "dense"
    assert eng.apply_path(nz) == ("modal" if nz <= 446 else "dense")
    x, p = _rand(grid, 21)
    fixed = bcs.reference_cpu(*grid, {"fixed_face": ["x_min", "y_max"]})[1] if masked else None
    m = _cuda(bcs.node_mask(*grid, fixed)) if masked else None
    lw = L.make_law("modified", 3.0)
    ym = eng.apply(grid, lw, _cuda(x), _cuda(p, torch.float32), m).cpu().numpy()
    yd = dense.apply(grid, lw, _cuda(x), _cuda(p, torch.float32), m).cpu().numpy()
    ref = O.apply(grid, O.ke_quadrature(), O.moduli(x.astype(np.float64), _mat("modified")), p,
                  bcs.dof_mask(*grid, fixed) if masked else None)
    np.testing.assert_allclose(ym, ref, rtol=0, atol=2e-6 * np.abs(ref).max())
    np.testing.assert_allclose(yd, ref, rtol=0, atol=2e-6 * np.abs(ref).max())


def test_pcg_dense_path_matches_modal_path(eng):
    grid = (20, 10, 14)
    f, fixed, x = _problem(grid)
    m = _cuda(bcs.node_mask(*grid, fixed))
    lw = L.make_law("modified", 3.0)
    out = []
    for e in (eng, Engine(ke=_perturbed_ke())):
        u = torch.zeros(n_dof(grid), dtype=torch.float64, device="cuda")
        st = e.solve(grid, lw, _cuda(x), _cuda(f), m, u, rtol=1e-8)
        assert st["status"] == L.GBS_OK
        out.append(u.cpu().numpy())
    np.testing.assert_allclose(out[0], out[1], rtol=0, atol=1e-6 * np.abs(out[1]).max())


@pytest.mark.parametrize("grid", [(5, 4, 3), (17, 9, 37)])
def test_apply_literal_reference_ke(grid, ke_lit):
    """Non-symmetric, translation-carrying reference table: the non-subtracting kernel."""
    e = Engine(ke=ke_lit)
    x, p = _rand(grid, 7)
    E = O.moduli(x.astype(np.float64), _mat("ref"))
    ref = O.apply(grid, ke_lit, E, p)
    lw = L.make_law("ref", 3.0)
    y64 = e.apply(grid, lw, _cuda(x), _cuda(p)).cpu().numpy()
    np.testing.assert_allclose(y64, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    y32 = e.apply(grid, lw, _cuda(x), _cuda(p, torch.float32)).cpu().numpy()
    np.testing.assert_allclose(y32, ref, rtol=0, atol=2e-6 * np.abs(ref).max())


@pytest.mark.parametrize("gname,grid", [("g543", (5, 4, 3)), ("g364", (3, 6, 4))])
@pytest.mark.parametrize("kname", ["lit", "spd"])
def test_apply_vs_reference_assembly(golden, gname, grid, kname):
    """Against K(x) p of the reference CPU COO assembly (which assembles Ke^T)."""
    g = golden("kernels")
    ke = golden("ke")["ke_reference" if kname == "lit" else "ke_quadrature"]
    e = Engine(ke=ke.T)
    y = e.apply(grid, L.make_law("ref", 3.0), _cuda(g[f"apply_{gname}_x"], torch.float32),
                _cuda(g[f"apply_{gname}_p"])).cpu().numpy()
    ref = g[f"apply_{gname}_{kname}_y"]
    # x is rounded to FP32 on the device: 1e-7 relative in E.
    np.testing.assert_allclose(y, ref, rtol=0, atol=1e-6 * np.abs(ref).max())


def test_apply_is_deterministic(eng):
    grid = (40, 24, 33)
    x, p = _rand(grid, 3)
    lw = L.make_law("modified", 3.0)
    a = eng.apply(grid, lw, _cuda(x), _cuda(p, torch.float32))
    b = eng.apply(grid, lw, _cuda(x), _cuda(p, torch.float32))
    assert torch.equal(a, b)


@pytest.mark.parametrize("grid", [(5, 4, 3), (33, 7, 5), (17, 9, 37)])
@pytest.mark.parametrize("law", ["ref", "modified"])
def test_sensitivity_vs_oracle(eng, grid, law):
    x, u = _rand(grid, 11)
    ke = O.ke_quadrature()
    ce, dc, tot = O.element_energy(grid, ke, x.astype(np.float64), u, _mat(law))
    en = torch.zeros((), dtype=torch.float64, device="cuda")
    cet = torch.empty(x.size, dtype=torch.float32, device="cuda")
    dcg = eng.sensitivity(grid, L.make_law(law, 3.0), _cuda(x), _cuda(u), ce=cet, energy=en)
    np.testing.assert_allclose(dcg.cpu().numpy(), dc, rtol=1e-6, atol=1e-7 * np.abs(dc).max())
    np.testing.assert_allclose(cet.cpu().numpy(), ce, rtol=1e-6, atol=1e-7 * np.abs(ce).max())
    assert en.item() == pytest.approx(tot, rel=1e-12)


@pytest.mark.parametrize("kname", ["lit", "spd"])
def test_sensitivity_vs_reference(golden, kname):
    g = golden("kernels")
    ke = golden("ke")["ke_reference" if kname == "lit" else "ke_quadrature"]
    e = Engine(ke=ke)
    grid = (6, 3, 3)
    dc = e.sensitivity(grid, L.make_law("ref", 3.0), _cuda(g["sens_x"], torch.float32),
                       _cuda(g[f"sens_{kname}_u"])).cpu().numpy()
    ref = g[f"sens_{kname}_dc"]
    np.testing.assert_allclose(dc, ref, rtol=2e-6, atol=1e-7 * np.abs(ref).max())


@pytest.mark.parametrize("rmin", [1.5, 2.0, 3.0])
def test_filter_vs_reference(eng, golden, rmin):
    g = golden("kernels")
    t = f"filter_r{rmin}"
    grid = (7, 6, 5)
    hs = eng.filter_hs(grid, rmin)
    np.testing.assert_allclose(hs.cpu().numpy(), g[t + "_Hs"], rtol=1e-6)
    v = _cuda(g[t + "_v"], torch.float32)
    np.testing.assert_allclose(eng.filter(grid, rmin, v, hs).cpu().numpy(), g[t + "_fwd"], rtol=1e-6)
    np.testing.assert_allclose(eng.filter(grid, rmin, v, None).cpu().numpy(), g[t + "_fwd"], rtol=1e-6)
    np.testing.assert_allclose(eng.filter(grid, rmin, v, hs, transpose=True).cpu().numpy(), g[t + "_adj"], rtol=1e-6)


@pytest.mark.parametrize("grid", [(33, 7, 5), (1, 1, 1), (12, 30, 9)])
@pytest.mark.parametrize("rmin", [1.5, 2.0, 3.0, 4.5])
def test_filter_vs_oracle(eng, grid, rmin):
    v = np.random.default_rng(5).uniform(0, 1, np.prod(grid))
    hs = O.filter_hs(grid, rmin)
    for tr in (False, True):
        ref = O.density_filter(grid, rmin, v, hs, transpose=tr)
        got = eng.filter(grid, rmin, _cuda(v, torch.float32), eng.filter_hs(grid, rmin), transpose=tr)
        np.testing.assert_allclose(got.cpu().numpy(), ref, rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("rmin", [1.5, 2.0])
@pytest.mark.parametrize("vf", [0.3, 0.5])
@pytest.mark.parametrize("pres", [False, True])
def test_oc_vs_reference(eng, golden, rmin, vf, pres):
    g = golden("kernels")
    grid = (6, 5, 4)
    p = _cuda(g["oc_pres"].astype(np.uint8)) if pres else None
    xn, xp = eng.oc(grid, rmin, vf, _cuda(g["oc_x"], torch.float32), _cuda(g["oc_dc"], torch.float32), p)
    tag = ("ocp" if pres else "oc") + f"_r{rmin}_v{vf}"
    np.testing.assert_allclose(xn.cpu().numpy(), g[tag + "_x"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(xp.cpu().numpy(), g[tag + "_xphys"], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("rmin", [1.5, 2.0])
def test_oc_gpu_variant(eng, golden, rmin):
    g = golden("kernels")
    if f"ocgpu_r{rmin}_x" not in g.files:
        pytest.skip("no SIMPSolverGPU fixture")
    xn, xp = eng.oc((6, 5, 4), rmin, 0.3, _cuda(g["oc_x"], torch.float32), _cuda(g["oc_dc"], torch.float32),
                    None, L.OC_GPU)
    np.testing.assert_allclose(xn.cpu().numpy(), g[f"ocgpu_r{rmin}_x"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(xp.cpu().numpy(), g[f"ocgpu_r{rmin}_xphys"], rtol=1e-5, atol=1e-6)


def test_oc_large_vs_oracle(eng):
    grid = (40, 20, 24)
    rng = np.random.default_rng(9)
    x = rng.uniform(0.01, 1, np.prod(grid))
    dc = -rng.gamma(2.0, 1.0, x.size) * 10 ** rng.uniform(-3, 0, x.size)
    pres = (rng.random(x.size) < 0.05).astype(np.uint8)
    for variant_o, variant_l in ((O.OC_CPU, L.OC_CPU), (O.OC_GPU, L.OC_GPU)):
        xn_o, xp_o, it = O.oc(grid, 2.0, x.astype(np.float32), dc.astype(np.float32), 0.3, pres, variant=variant_o)
        xn, xp = eng.oc(grid, 2.0, 0.3, _cuda(x, torch.float32), _cuda(dc, torch.float32), _cuda(pres), variant_l)
        lam, steps = eng.oc_result()
        assert steps == it
        np.testing.assert_allclose(xn.cpu().numpy(), xn_o, rtol=1e-4, atol=1e-5)
        np.testing.assert_allclose(xp.cpu().numpy(), xp_o, rtol=1e-4, atol=1e-5)


def _problem(grid, case="cantilever", law="modified", seed=0):
    """Load case and seeded random densities in [0.05, 1)."""
    f, fixed = bcs.LOAD_CASES[case](*grid)
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.05, 1.0, np.prod(grid)).astype(np.float32)
    return f, fixed, x


@pytest.mark.parametrize("grid", [(12, 6, 6), (20, 10, 14)])
def test_pcg_f32_vs_oracle(eng, grid):
    f, fixed, x = _problem(grid)
    ke = O.ke_quadrature()
    E = O.moduli(x.astype(np.float64), _mat("modified"))
    dm = bcs.dof_mask(*grid, fixed)
    uref, _, _ = O.pcg(grid, ke, E, f, dm, tol=1e-13)
    u = torch.zeros(n_dof(grid), dtype=torch.float32, device="cuda")
    st = eng.pcg(grid, L.make_law("modified", 3.0), _cuda(x), _cuda(f, torch.float32),
                 _cuda(bcs.node_mask(*grid, fixed)), u, rtol=1e-5, max_iter=5000)
    assert st["status"] == L.GBS_OK and st["relres"] < 1e-5
    np.testing.assert_allclose(u.cpu().numpy(), uref, rtol=0, atol=1e-3 * np.abs(uref).max())


@pytest.mark.parametrize("grid,case", [((12, 6, 6), "cantilever"), ((16, 16, 10), "top_patch"),
                                       ((10, 8, 8), "torsion"), ((24, 8, 8), "edge_line")])
@pytest.mark.parametrize("law", ["ref", "modified"])
def test_solve_refined_vs_oracle(eng, grid, case, law):
    """FP32 PCG + FP64 defect correction to rtol 1e-8: compliance within 1e-6 of FP64."""
    f, fixed, x = _problem(grid, case)
    ke = O.ke_quadrature()
    E = O.moduli(x.astype(np.float64), _mat(law))
    uref, _, _ = O.pcg(grid, ke, E, f, bcs.dof_mask(*grid, fixed), tol=1e-13)
    u = torch.zeros(n_dof(grid), dtype=torch.float64, device="cuda")
    st = eng.solve(grid, L.make_law(law, 3.0), _cuda(x), _cuda(f), _cuda(bcs.node_mask(*grid, fixed)), u, rtol=1e-8)
    assert st["status"] == L.GBS_OK and st["relres"] <= 1e-8, st
    ug = u.cpu().numpy()
    c_ref = float(f @ uref)
    assert float(f @ ug) == pytest.approx(c_ref, rel=1e-6)
    np.testing.assert_allclose(ug, uref, rtol=0, atol=1e-5 * np.abs(uref).max())


@pytest.mark.parametrize("grid,case", [((16, 16, 10), "top_patch"), ((48, 24, 24), "cantilever"),
                                       ((64, 64, 64), "top_patch")])
def test_double_float_residual_certifies_fp64(eng, grid, case):
    """At rtol >= 1e-9 the outer residual's element products run in double-float: the relres
    a solve reports agrees with the FP64 residual of the returned u (FP64 apply) to 1e-11."""
    f, fixed, x = _problem(grid, case)
    lw = L.make_law("modified", 3.0)
    m = _cuda(bcs.node_mask(*grid, fixed))
    xd = _cuda(x)
    u = torch.zeros(n_dof(grid), dtype=torch.float64, device="cuda")
    st = eng.solve(grid, lw, xd, _cuda(f), m, u, rtol=1e-8)
    assert st["status"] == L.GBS_OK and st["relres"] <= 1e-8, st
    y = eng.apply(grid, lw, xd, u, m)
    fixed_dof = _cuda(bcs.dof_mask(*grid, fixed).astype(bool))
    fd = _cuda(f)
    r = torch.where(fixed_dof, 0.0, fd - y)
    rel64 = (r.norm() / torch.where(fixed_dof, 0.0, fd).norm()).item()
    assert abs(rel64 - st["relres"]) <= 1e-11, (rel64, st["relres"])
    # the FP64 form on request: the same certificate, to FP64 rounding
    u2 = torch.zeros_like(u)
    st2 = eng.solve(grid, lw, xd, _cuda(f), m, u2, rtol=1e-8, residual_fp64=True)
    assert st2["status"] == L.GBS_OK and st2["relres"] <= 1e-8, st2
    r2 = torch.where(fixed_dof, 0.0, fd - eng.apply(grid, lw, xd, u2, m))
    assert abs((r2.norm() / torch.where(fixed_dof, 0.0, fd).norm()).item() - st2["relres"]) <= 1e-13


@pytest.mark.parametrize("grid,case", [((12, 6, 6), "cantilever"), ((24, 12, 12), "top_patch")])
@pytest.mark.parametrize("law", ["ref", "modified"])
def test_sensitivity_double_float_vs_fp64(eng, grid, case, law):
    """The double-float sensitivity (workspace with room for the split of u) against the FP64
    pass (a workspace sized for the energy sum only) on a converged displacement: dc and ce
    to FP32 rounding, the energy to 1e-10. The double-float modes carry about 2^-46 of the
    element's displacement magnitudes, which exceed its strain modes by up to the grid length
    (2e-12 relative energy difference measured on the 12x6x6 cantilever)."""
    import ctypes as C

    from genpipeline_gb300.engine import _p, _stream

    f, fixed, x = _problem(grid, case)
    lw = L.make_law(law, 3.0)
    xd = _cuda(x)
    u = torch.zeros(n_dof(grid), dtype=torch.float64, device="cuda")
    eng.solve(grid, lw, xd, _cuda(f), _cuda(bcs.node_mask(*grid, fixed)), u, rtol=1e-8)
    ne = int(np.prod(grid))
    out = {}
    for full in (True, False):
        nb = eng.lib.gbsimp_sensitivity_ws_bytes(*grid) if full else 256 + 4096 * 32
        ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
        dc = torch.empty(ne, dtype=torch.float32, device="cuda")
        ce = torch.empty(ne, dtype=torch.float32, device="cuda")
        en = torch.zeros((), dtype=torch.float64, device="cuda")
        L.check(eng.lib.gbsimp_sensitivity(eng.ctx, *grid, C.byref(lw), _p(xd), _p(u), _p(dc), _p(ce), _p(en),
                                           _p(ws), nb, _stream()))
        out[full] = (dc.cpu().numpy(), ce.cpu().numpy(), en.item())
    (dc1, ce1, e1), (dc0, ce0, e0) = out[True], out[False]
    np.testing.assert_allclose(dc1, dc0, rtol=2e-7, atol=1e-9 * np.abs(dc0).max())
    np.testing.assert_allclose(ce1, ce0, rtol=2e-7, atol=1e-9 * np.abs(ce0).max())
    assert e1 == pytest.approx(e0, rel=1e-10)


def test_device_loop_and_host_loop_agree_bitwise(eng):
    """The graph WHILE loop and the host-launched (profiled) loop run the same kernels in the
    same order: identical bits, identical iteration counts."""
    grid = (24, 12, 12)
    f, fixed, x = _problem(grid, "top_patch")
    m = _cuda(bcs.node_mask(*grid, fixed))
    lw = L.make_law("modified", 3.0)
    res = []
    for prof in (False, True, False):
        u = torch.zeros(n_dof(grid), dtype=torch.float64, device="cuda")
        st = eng.solve(grid, lw, _cuda(x), _cuda(f), m, u, rtol=1e-8, profile=prof)
        assert st["status"] == L.GBS_OK
        res.append((u.cpu().numpy(), st["iterations"]))
        if prof:
            assert st["apply_launches"] == st["iterations"] and st["apply_seconds"] > 0
    assert res[0][1] == res[1][1] == res[2][1]
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][0], res[2][0])


@pytest.mark.parametrize("grid,case", [((24, 12, 12), "top_patch"), ((64, 32, 32), "cantilever"),
                                       ((40, 20, 100), "edge_line")])
def test_fused_persistent_pcg_matches_graph_loop(eng, grid, case):
    """One cooperative launch for the whole inner PCG (grid barriers) against the graph loop
    of one launch per iteration: same solution to the solve tolerance, iteration counts within
    12%. The FP32 iterates round differently: the partial sums are grouped differently, the
    graph loop's x segments add the two halves of their shared node planes where the
    persistent kernel computes a halo element plane, and the graph loop starts from a start
    pass where the persistent kernel uses the setup's apply. Where an inner solve stops
    depends on that rounding, so the totals of several outer rounds spread: measured 383
    against 417 (24x12x12), 1663 against 1614 (64^3)."""
    f, fixed, x = _problem(grid, case)
    m = _cuda(bcs.node_mask(*grid, fixed))
    lw = L.make_law("modified", 3.0)
    out = {}
    for fused in (False, True):
        u = torch.zeros(n_dof(grid), dtype=torch.float64, device="cuda")
        st = eng.solve(grid, lw, _cuda(x), _cuda(f), m, u, rtol=1e-8, fused=fused)
        assert st["status"] == L.GBS_OK and st["relres"] <= 1e-8, st
        out[fused] = (u.cpu().numpy(), st["iterations"])
    np.testing.assert_allclose(out[True][0], out[False][0], rtol=0, atol=1e-6 * np.abs(out[False][0]).max())
    assert abs(out[True][1] - out[False][1]) <= max(5, 0.12 * out[False][1])


def test_fused_pcg_is_deterministic(eng):
    grid = (32, 16, 16)
    f, fixed, x = _problem(grid)
    m = _cuda(bcs.node_mask(*grid, fixed))
    lw = L.make_law("modified", 3.0)
    res = []
    for _ in range(2):
        u = torch.zeros(n_dof(grid), dtype=torch.float64, device="cuda")
        eng.solve(grid, lw, _cuda(x), _cuda(f), m, u, rtol=1e-8, fused=True)
        res.append(u.cpu().numpy())
    assert np.array_equal(res[0], res[1])


def test_time_pcg_apply(eng):
    grid = (32, 16, 16)
    f, fixed, x = _problem(grid)
    sec = eng.time_pcg_apply(grid, L.make_law("modified", 3.0), _cuda(x), _cuda(bcs.node_mask(*grid, fixed)), reps=10)
    assert 0 < sec < 1e-2


def test_solve_warm_start_and_zero_load(eng):
    grid = (10, 6, 6)
    f, fixed, x = _problem(grid)
    m = _cuda(bcs.node_mask(*grid, fixed))
    lw = L.make_law("modified", 3.0)
    u = torch.zeros(n_dof(grid), dtype=torch.float64, device="cuda")
    s1 = eng.solve(grid, lw, _cuda(x), _cuda(f), m, u)
    s2 = eng.solve(grid, lw, _cuda(x), _cuda(f), m, u)  # warm start at the solution
    assert s2["iterations"] == 0 and s2["relres"] <= 1e-8 and s1["iterations"] > 0
    z = torch.zeros(n_dof(grid), dtype=torch.float64, device="cuda")
    uz = torch.ones(n_dof(grid), dtype=torch.float64, device="cuda")
    s3 = eng.solve(grid, lw, _cuda(x), z, m, uz)
    assert s3["status"] == L.GBS_OK and torch.count_nonzero(uz).item() == 0


@pytest.mark.parametrize("fused", [False, True])
def test_solve_inner_start_stop_rules(eng, fused):
    """The inner solves of the graph loop start with a start pass whose sums the next launch
    folds into alpha_0 (the persistent form keeps the setup kernels); both stop the same way.
    An iteration cap of 5 ends the inner solve after exactly 5 iterations and the outer loop
    with ENOTCONV; an inner tolerance above 1 is met by x0 = 0 at once, so no iteration runs,
    u stays zero and the outer loop ends at its round cap."""
    grid = (12, 6, 6)
    f, fixed, x = _problem(grid)
    m = _cuda(bcs.node_mask(*grid, fixed))
    lw = L.make_law("modified", 3.0)
    u = torch.zeros(n_dof(grid), dtype=torch.float64, device="cuda")
    st = eng.solve(grid, lw, _cuda(x), _cuda(f), m, u, max_iter=5, fused=fused)
    assert st["status"] == L.GBS_ENOTCONV and st["iterations"] == 5, st
    assert 0.0 < st["relres"] < 1.0 and torch.isfinite(u).all()
    u.zero_()
    st = eng.solve(grid, lw, _cuda(x), _cuda(f), m, u, inner_rtol=2.0, max_outer=3, fused=fused)
    assert st["status"] == L.GBS_ENOTCONV and st["iterations"] == 0, st
    assert torch.count_nonzero(u).item() == 0


def test_pcg_breakdown_and_cap_are_statuses(eng):
    grid = (8, 4, 4)
    f, fixed, x = _problem(grid)
    lw = L.make_law("modified", 3.0)
    u = torch.zeros(n_dof(grid), dtype=torch.float32, device="cuda")
    st = eng.pcg(grid, lw, _cuda(x), _cuda(f, torch.float32), _cuda(bcs.node_mask(*grid, fixed)), u, rtol=1e-12,
                 max_iter=3)
    assert st["status"] == L.GBS_ENOTCONV and st["iterations"] == 3
    # A NaN density must come back as a status, not as a fault or a hang.
    xn = x.copy()
    xn[5] = np.nan
    u.zero_()
    st = eng.pcg(grid, lw, _cuda(xn), _cuda(f, torch.float32), _cuda(bcs.node_mask(*grid, fixed)), u, rtol=1e-6,
                 max_iter=50)
    assert st["status"] in (L.GBS_ENONFINITE, L.GBS_EBREAKDOWN)


def test_dot64(eng):
    a = torch.randn(1_000_003, dtype=torch.float64, device="cuda")
    b = torch.randn(1_000_003, dtype=torch.float64, device="cuda")
    assert eng.dot64(a, b).item() == pytest.approx(float(a.cpu().numpy() @ b.cpu().numpy()), rel=1e-12)


def test_library_rejects_bad_arguments(eng):
    lw = L.make_law("ref", 3.0)
    with pytest.raises(L.GbsimpError):
        eng.filter((4, 4, 4), 7.5, torch.zeros(64, device="cuda"))
    with pytest.raises(L.GbsimpError):
        L.check(eng.lib.gbsimp_apply_f32(eng.ctx, 0, 1, 1, lw, None, None, None, None, None))


def test_warm_start_extrapolation(eng):
    rng = np.random.default_rng(4)
    a, b = rng.standard_normal(1000), rng.standard_normal(1000)
    u, up = _cuda(a), _cuda(b)
    eng.warm_start(u, up, 0.5)
    np.testing.assert_allclose(u.cpu().numpy(), a + 0.5 * (a - b), rtol=1e-15, atol=1e-15)
    assert np.array_equal(up.cpu().numpy(), a)
