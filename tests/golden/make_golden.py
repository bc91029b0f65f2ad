"""Generate the golden fixtures for the SIMP hot path by running the reference itself.

This script imports the reference package ``genpipeline`` (a checkout given by
``--reference`` or the ``GENPIPELINE_REFERENCE`` environment variable) and records what its own CPU code returns
on small seeded inputs. The GPU tests and the oracle tests compare against these
``.npz`` files; nothing at test time imports the reference.

Recorded (all FP64):

* ``ke.npz``            the reference's literal element stiffness
                        (``genpipeline/topology/simp_solver.py:284-1543``) and the
                        quadrature stiffness this script derives (the SPD matrix that is
                        injected into the reference solver for the SIMP runs below).
* ``kernels.npz``       edof map (``simp_solver.py:251-282``), filter ``H@v``/``Hs``/
                        ``H.T@(v/Hs)`` (``:221-223``, ``:1545-1567``), ``K(x)@p`` through
                        the reference COO assembly (``:200-205``), ``u``/``dc`` of
                        ``SIMPSolver._sensitivity`` (``:195-219``), OC (``:225-249``) and the
                        ``SIMPSolverGPU._oc_update`` variant (``simp_solver_gpu.py:801-841``).
* ``bcs.npz``           ``SIMPSolver._get_bcs`` (``simp_solver.py:81-157``) and
                        ``SIMPSolverGPU._get_bcs`` (``simp_solver_gpu.py:138-311``) for a
                        set of boundary-condition dicts.
* ``simp_small.npz``    whole ``SIMPSolver.run`` trajectories (``:56-79``) on small grids
                        with the SPD stiffness injected.
* ``simp_c0.npz``       (``--c0``, ~7 min) the 32x16x16, volfrac 0.3, rmin 1.5, penal 3,
                        50-iteration ``SIMPSolver.run`` with the SPD stiffness injected.
* ``voxel.npz``         the evaluator's input step as ``VoxelFEMEvaluator.evaluate`` runs
                        it (``genpipeline/fem/voxel_fem.py:457-462``):
                        ``scipy.ndimage.zoom(v, zoom, order=1)`` then the reference's
                        ``pipeline_utils.smooth_voxels`` (``:55-76``), on float32 grids
                        (the decoder's dtype). Inputs are seeded ``PCG64`` uniforms.
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def quadrature_ke(nu: float = 0.3, e0: float = 1.0) -> np.ndarray:
    """Unit-cube trilinear hexahedron stiffness by 2x2x2 Gauss quadrature of B^T D B.

    Node order (x,y,z): (0,0,0),(1,0,0),(1,1,0),(0,1,0),(0,0,1),(1,0,1),(1,1,1),(0,1,1);
    DOF 3a+c. Engineering shear strains ordered (xy, yz, zx).
    """
    lam = e0 * nu / ((1 + nu) * (1 - 2 * nu))
    mu = e0 / (2 * (1 + nu))
    d = np.zeros((6, 6))
    d[:3, :3] = lam
    for i in range(3):
        d[i, i] = lam + 2 * mu
        d[3 + i, 3 + i] = mu
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
               (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    g = [0.5 - 0.5 / np.sqrt(3.0), 0.5 + 0.5 / np.sqrt(3.0)]
    ke = np.zeros((24, 24))
    for qx, qy, qz in itertools.product(g, g, g):
        b = np.zeros((6, 24))
        for a, (cx, cy, cz) in enumerate(corners):
            fx = qx if cx else 1 - qx
            fy = qy if cy else 1 - qy
            fz = qz if cz else 1 - qz
            dx = (1 if cx else -1) * fy * fz
            dy = fx * (1 if cy else -1) * fz
            dz = fx * fy * (1 if cz else -1)
            b[0, 3 * a] = dx
            b[1, 3 * a + 1] = dy
            b[2, 3 * a + 2] = dz
            b[3, 3 * a], b[3, 3 * a + 1] = dy, dx
            b[4, 3 * a + 1], b[4, 3 * a + 2] = dz, dy
            b[5, 3 * a], b[5, 3 * a + 2] = dz, dx
        ke += b.T @ d @ b / 8.0
    return 0.5 * (ke + ke.T)


def _import_reference(path: str):
    sys.path.insert(0, path)
    import genpipeline.topology.simp_solver as ss  # noqa: E402
    return ss


class _Recorder:
    """Wraps the module-level ``spsolve`` of the reference to capture its solutions."""

    def __init__(self, ss):
        self.ss = ss
        self.orig = ss.spsolve
        self.last = None

    def __enter__(self):
        def rec(a, b):
            x = self.orig(a, b)
            self.last = np.array(x, dtype=np.float64)
            return x
        self.ss.spsolve = rec
        return self

    def __exit__(self, *exc):
        self.ss.spsolve = self.orig


def _solver(ss, nx, ny, nz, penal, rmin, ke=None, bcs=None, preserved=None):
    s = ss.SIMPSolver(nx, ny, nz, penal=penal, rmin=rmin, boundary_conditions=bcs,
                      preserved_mask=preserved)
    if ke is not None:
        s.Ke = ke.copy()
    return s


def make_ke(ss, out):
    ke_lit = np.asarray(ss.SIMPSolver._get_Ke(0.3), dtype=np.float64)
    np.savez_compressed(out, ke_reference=ke_lit, ke_quadrature=quadrature_ke(0.3))


def make_kernels(ss, out):
    rng = np.random.default_rng(20261203)
    ke_lit = np.asarray(ss.SIMPSolver._get_Ke(0.3), dtype=np.float64)
    ke_spd = quadrature_ke(0.3)
    rec = {}
    nx, ny, nz = 5, 4, 3
    s = _solver(ss, nx, ny, nz, 3.0, 1.5)
    rec["edof_5x4x3"] = s._edof_mat.astype(np.int64)
    # filters at three radii on a 7x6x5 grid
    for rmin in (1.5, 2.0, 3.0):
        H, Hs = ss.SIMPSolver._build_filter(7, 6, 5, rmin)
        v = rng.random(7 * 6 * 5)
        tag = f"filter_r{rmin}"
        rec[tag + "_v"] = v
        rec[tag + "_Hs"] = np.asarray(Hs, dtype=np.float64)
        rec[tag + "_fwd"] = np.asarray(H @ v).ravel() / Hs
        rec[tag + "_adj"] = np.asarray(H.T @ (v / Hs)).ravel()
    # K(x) p through the reference COO assembly, both element stiffnesses
    for gname, (gx, gy, gz) in {"g543": (5, 4, 3), "g364": (3, 6, 4)}.items():
        s = _solver(ss, gx, gy, gz, 3.0, 1.5)
        ne = gx * gy * gz
        ndof = 3 * (gx + 1) * (gy + 1) * (gz + 1)
        x = rng.uniform(0.0, 1.0, ne)
        x[:3] = [0.0, 5e-4, 1.0]
        p = rng.standard_normal(ndof)
        rec[f"apply_{gname}_x"] = x
        rec[f"apply_{gname}_p"] = p
        for kname, ke in (("lit", ke_lit), ("spd", ke_spd)):
            sK = (ke.ravel()[np.newaxis, :] * (np.maximum(x, 1e-3) ** 3.0)[:, np.newaxis]).ravel()
            K = ss.coo_matrix((sK, (s._iK, s._jK)), shape=(ndof, ndof)).tocsc()
            rec[f"apply_{gname}_{kname}_y"] = K @ p
    # _sensitivity: u (via spsolve) and dc, both element stiffnesses, default BCs
    nx, ny, nz = 6, 3, 3
    xs = rng.uniform(0.05, 1.0, nx * ny * nz)
    rec["sens_x"] = xs
    for kname, ke in (("lit", ke_lit), ("spd", ke_spd)):
        s = _solver(ss, nx, ny, nz, 3.0, 1.5, ke=ke)
        with _Recorder(ss) as r:
            dc = s._sensitivity(xs, 1.0)
        f, fixed = s._get_bcs(1.0)
        u = np.zeros_like(f)
        free = np.setdiff1d(np.arange(f.size), fixed)
        u[free] = r.last
        rec[f"sens_{kname}_u"] = u
        rec[f"sens_{kname}_dc"] = np.asarray(dc, dtype=np.float64)
        rec[f"sens_{kname}_dcf"] = s._filter_dc(dc)
    # OC update (CPU variant) with and without a preserved mask
    nx, ny, nz = 6, 5, 4
    ne = nx * ny * nz
    x = rng.uniform(0.0, 1.0, ne)
    xp = rng.uniform(0.0, 1.0, ne)
    dc = -rng.gamma(2.0, 1.0, ne) * 10 ** rng.uniform(-3, 1, ne)
    dc[:2] = [0.0, 1e-3]  # a zero and a positive sensitivity hit the sqrt floor
    pres = rng.random(ne) < 0.1
    rec["oc_x"], rec["oc_xphys"], rec["oc_dc"], rec["oc_pres"] = x, xp, dc, pres
    for rmin in (1.5, 2.0):
        for vf in (0.3, 0.5):
            s = _solver(ss, nx, ny, nz, 3.0, rmin)
            xn, xpn = s._oc_update(x.copy(), xp.copy(), dc.copy(), vf)
            rec[f"oc_r{rmin}_v{vf}_x"], rec[f"oc_r{rmin}_v{vf}_xphys"] = xn, xpn
            s = _solver(ss, nx, ny, nz, 3.0, rmin, preserved=pres.reshape(nx, ny, nz))
            xn, xpn = s._oc_update(x.copy(), xp.copy(), dc.copy(), vf)
            rec[f"ocp_r{rmin}_v{vf}_x"], rec[f"ocp_r{rmin}_v{vf}_xphys"] = xn, xpn
    # SIMPSolverGPU._oc_update (runs on the CPU through torch sparse)
    try:
        import torch
        import genpipeline.topology.simp_solver_gpu as sg
        for rmin in (1.5, 2.0):
            g = sg.SIMPSolverGPU(nx, ny, nz, penal=3.0, rmin=rmin, device="cpu",
                                 dtype=torch.float64)
            xn, xpn = g._oc_update(torch.from_numpy(x.copy()), torch.from_numpy(xp.copy()),
                                   torch.from_numpy(dc.copy()), 0.3)
            rec[f"ocgpu_r{rmin}_x"] = xn.numpy()
            rec[f"ocgpu_r{rmin}_xphys"] = xpn.numpy()
    except Exception as exc:  # pragma: no cover - recorded for the log only
        print("SIMPSolverGPU OC skipped:", exc)
    np.savez_compressed(out, **rec)


BCS_CASES = {
    "default": None,
    "faces_list": {"fixed_face": ["x_min", "y_min"], "load_face": "x_max", "load_dof": 1},
    "center": {"fixed_face": ["z_min"], "load_face": "center", "load_dof": 2},
    "top": {"fixed_face": "z_min", "load_face": "top", "load_dof": 2},
    "x_max_offset": {"fixed_face": "x_min", "load_face": "x_max_offset", "load_dof": 2},
    "multi": {"fixed_face": "x_min", "load_face": "x_max", "load_dof": [1, 2],
              "multi_load": True},
    "z_max_face": {"fixed_face": "z_max", "load_face": "z_min", "load_dof": 0},
    "y_faces": {"fixed_face": "y_min", "load_face": "y_max", "load_dof": 1},
    "all_fixed_load": {"fixed_face": ["x_max", "x_min"], "load_face": "x_max", "load_dof": 2},
}

GPU_BCS_CASES = {
    "default": None,
    "y_faces": {"fixed_face": "y_min", "load_face": "y_max", "load_dof": 1},
    "multi_pos": {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2,
                  "multi_load": True, "load_positions": ["top", "mid", "bottom", "other"]},
    "grid": {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2,
             "multi_load": True, "load_pattern": "grid"},
    "same_face": {"fixed_face": "x_max", "load_face": "x_max", "load_dof": 2},
}


def make_bcs(ss, out):
    rec = {"cases": json.dumps(BCS_CASES), "gpu_cases": json.dumps(GPU_BCS_CASES)}
    for (gx, gy, gz) in ((6, 4, 5), (7, 3, 4)):
        for name, bcs in BCS_CASES.items():
            s = _solver(ss, gx, gy, gz, 3.0, 1.5, bcs=bcs)
            f, fixed = s._get_bcs(2.5)
            rec[f"cpu_{gx}{gy}{gz}_{name}_f"] = np.asarray(f, dtype=np.float64)
            rec[f"cpu_{gx}{gy}{gz}_{name}_fixed"] = np.unique(np.asarray(fixed, dtype=np.int64))
    try:
        import torch
        import genpipeline.topology.simp_solver_gpu as sg
        for (gx, gy, gz) in ((6, 4, 5), (7, 3, 8)):
            for name, bcs in GPU_BCS_CASES.items():
                g = sg.SIMPSolverGPU(gx, gy, gz, penal=3.0, rmin=1.5, boundary_conditions=bcs,
                                     device="cpu", dtype=torch.float64)
                f, fixed = g._get_bcs(2.5)
                rec[f"gpu_{gx}{gy}{gz}_{name}_f"] = f.numpy().astype(np.float64)
                rec[f"gpu_{gx}{gy}{gz}_{name}_fixed"] = np.unique(fixed.numpy().astype(np.int64))
    except Exception as exc:  # pragma: no cover
        print("SIMPSolverGPU BCs skipped:", exc)
    np.savez_compressed(out, **rec)


SMALL_RUNS = {
    "cantilever_12x6x6": dict(grid=(12, 6, 6), penal=3.0, rmin=1.5, volfrac=0.3, iters=12,
                               bcs=None, preserved=None, force=1.0),
    "bridge_10x4x6_r2": dict(grid=(10, 4, 6), penal=3.0, rmin=2.0, volfrac=0.4, iters=8,
                              bcs={"fixed_face": ["x_min", "x_max"], "load_face": "top",
                                   "load_dof": 2}, preserved=None, force=2.0),
    "preserved_8x5x5": dict(grid=(8, 5, 5), penal=3.0, rmin=1.5, volfrac=0.35, iters=6,
                            bcs={"fixed_face": "z_min", "load_face": "center",
                                 "load_dof": 2}, preserved="corner", force=1.0),
}


def make_simp_small(ss, out):
    ke_spd = quadrature_ke(0.3)
    rec = {"cases": json.dumps(SMALL_RUNS)}
    orig = ss.SIMPSolver._get_Ke
    ss.SIMPSolver._get_Ke = staticmethod(lambda nu=0.3: quadrature_ke(nu))
    try:
        for name, c in SMALL_RUNS.items():
            nx, ny, nz = c["grid"]
            pres = None
            if c["preserved"] == "corner":
                pres = np.zeros((nx, ny, nz), dtype=bool)
                pres[nx - 2:, :2, nz - 2:] = True
                rec[name + "_preserved"] = pres.ravel()
            s = ss.SIMPSolver(nx, ny, nz, penal=c["penal"], rmin=c["rmin"],
                              boundary_conditions=c["bcs"], preserved_mask=pres)
            assert np.allclose(s.Ke, ke_spd)
            xphys = s.run(volfrac=c["volfrac"], n_iters=c["iters"], force_mag=c["force"])
            rec[name + "_xphys"] = np.asarray(xphys, dtype=np.float64).ravel()
            rec[name + "_compliance"] = np.float64(s.last_compliance)
    finally:
        ss.SIMPSolver._get_Ke = orig
    np.savez_compressed(out, **rec)


def make_c0(ss, out):
    orig = ss.SIMPSolver._get_Ke
    ss.SIMPSolver._get_Ke = staticmethod(lambda nu=0.3: quadrature_ke(nu))
    try:
        s = ss.SIMPSolver(32, 16, 16, penal=3.0, rmin=1.5)
        t0 = time.time()
        xphys = s.run(volfrac=0.3, n_iters=50, force_mag=1.0)
        dt = time.time() - t0
    finally:
        ss.SIMPSolver._get_Ke = orig
    np.savez_compressed(out, xphys=np.asarray(xphys, dtype=np.float64).ravel(),
                        compliance=np.float64(s.last_compliance), seconds=np.float64(dt),
                        iters=np.int64(50))
    print(f"C0: compliance {s.last_compliance:.10f} in {dt:.1f} s")


VOXEL_CASES = [  # (name, input shape, seed, zoom)
    ("z16", (16, 16, 16), 1, 0.5),
    ("z64", (64, 64, 64), 2, 0.5),
    ("s_only", (12, 10, 9), 3, 1.0),
    ("z_odd", (20, 17, 9), 4, 0.5),
]


def voxel_input(shape, seed) -> np.ndarray:
    return np.random.Generator(np.random.PCG64(seed)).random(shape, dtype=np.float32)


def make_voxel(path):
    from scipy.ndimage import zoom

    from genpipeline.pipeline_utils import smooth_voxels

    out = {}
    for name, shape, seed, z in VOXEL_CASES:
        v = voxel_input(shape, seed)
        if z != 1.0:
            v = zoom(v, z, order=1)
        r = smooth_voxels(v)
        out[f"{name}_out"] = np.asarray(r, dtype=np.float32)
        if int(np.prod(shape)) <= 16 ** 3:
            out[f"{name}_in"] = voxel_input(shape, seed)
    np.savez_compressed(path, **out)
    print("wrote", path, {k: v.shape for k, v in out.items()})


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("GENPIPELINE_REFERENCE"),
                    required=os.environ.get("GENPIPELINE_REFERENCE") is None,
                    help="checkout of the reference repository (the directory holding genpipeline/)")
    ap.add_argument("--c0", action="store_true", help="also run the 50-iteration 32x16x16 case")
    ap.add_argument("--only-c0", action="store_true")
    ap.add_argument("--only-voxel", action="store_true", help="only the evaluator input step fixtures")
    a = ap.parse_args()
    ss = _import_reference(a.reference)
    if a.only_voxel:
        make_voxel(os.path.join(HERE, "voxel.npz"))
        return
    make_voxel(os.path.join(HERE, "voxel.npz"))
    if not a.only_c0:
        make_ke(ss, os.path.join(HERE, "ke.npz"))
        make_kernels(ss, os.path.join(HERE, "kernels.npz"))
        make_bcs(ss, os.path.join(HERE, "bcs.npz"))
        make_simp_small(ss, os.path.join(HERE, "simp_small.npz"))
    if a.c0 or a.only_c0:
        make_c0(ss, os.path.join(HERE, "simp_c0.npz"))


if __name__ == "__main__":
    main()
