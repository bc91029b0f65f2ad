"""SIMP trajectory fixtures of the benchmark configurations, from the FP64 oracle.

The oracle (``oracle/simp_oracle.c``) restates ``SIMPSolver.run``
(``genpipeline/topology/simp_solver.py:56-79``) and is pinned to the reference's own outputs
by ``tests/test_oracle_golden.py`` (50-iteration 32x16x16 run, small trajectories, filter,
OC, spsolve). The reference class itself cannot run these setups: it has no modified SIMP
law and no point load at (32, 8, 0) or top-patch traction, and at 64^3 its direct solve
takes about 9 h per iteration. So these fixtures come from the oracle, step by step:

* ``traj_c0.npz``  32x16x16, modified law (Emin 1e-9), x=0 clamped, unit -z point load at
                   node (32, 8, 0), volfrac 0.3, rmin 1.5, penal 3, 50 OC iterations.
* ``traj_c1.npz``  64^3, same law, z=0 clamped, -z traction of total 1 on the central 16x16
                   element patch of the top face, volfrac 0.25, rmin 2, 100 OC iterations.
* ``traj_c0ref.npz`` 32x16x16 with ``SIMPSolver``'s own law and boundary conditions, 50
                   iterations (its FP64 part reproduces the reference's recorded run).

Each holds, per OC iteration k: the objective c_k = f.u_k at the iteration's xPhys, the
bisection step count and mean(xPhys_{k+1}); and the final x, xPhys (float32) and the closing
compliance (``simp_solver.py:78``). The FP64 solves run to rtol 1e-11.

Drift study (stored beside it with the prefix ``drift_``): the same loop again with what a
single-precision implementation stores rounded to float32 (dc, filtered dc, x, xPhys) and
its solves stopped at rtol 1e-8, warm-started. Its distance from the FP64 trajectory is the
drift that FP32 storage alone causes, whatever the kernels: the GPU tests set their
tolerances from it.

Usage: ``python tests/golden/make_trajectories.py [--only c0|c0ref|c1] [--threads N]``.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from genpipeline_gb300 import bcs  # noqa: E402
from oracle import oracle as O  # noqa: E402

CASES = {
    "c0": dict(grid=(32, 16, 16), load="cantilever", law="modified", rmin=1.5, volfrac=0.3, iters=50),
    "c1": dict(grid=(64, 64, 64), load="top_patch", law="modified", rmin=2.0, volfrac=0.25, iters=100),
    # SIMPSolver's own defaults (reference law max(x, 1e-3)^3, x_min clamped, -z load at the
    # x_max face centre): the FP64 run equals tests/golden/simp_c0.npz, recorded from the
    # reference, to 1e-13; only its drift entries are new.
    "c0ref": dict(grid=(32, 16, 16), load="reference", law="ref", rmin=1.5, volfrac=0.3, iters=50),
}


def _load(case):
    if case["load"] == "reference":
        return bcs.reference_cpu(*case["grid"], None, 1.0)
    return bcs.LOAD_CASES[case["load"]](*case["grid"])


def _r32(a):
    return a.astype(np.float32).astype(np.float64)


def trajectory(case: dict, fp32_storage: bool, log=None):
    grid = case["grid"]
    f, fixed = _load(case)
    mask = bcs.dof_mask(*grid, fixed)
    mat = O.Material(case["law"], 3.0)
    ke = O.ke_quadrature()
    rmin, vf = case["rmin"], case["volfrac"]
    tol = 1e-8 if fp32_storage else 1e-11
    hs = O.filter_hs(grid, rmin)
    if fp32_storage:
        hs = _r32(hs)
    ne = int(np.prod(grid))
    x = np.full(ne, vf)
    if fp32_storage:
        x = _r32(x)
    xphys = x.copy()
    u = np.zeros_like(f)
    comp, steps, mean, pcg = [], [], [], []
    for k in range(case["iters"]):
        t = time.time()
        E = O.moduli(xphys, mat)
        u, its, _ = O.pcg(grid, ke, E, f, mask, u0=u, tol=tol)
        _, dc, _ = O.element_energy(grid, ke, xphys, u, mat)
        c = float(f @ u)
        if fp32_storage:
            dc = _r32(dc)
        dcf = O.density_filter(grid, rmin, dc, hs=hs, transpose=True)
        if fp32_storage:
            dcf = _r32(dcf)
        xn, xp, nb = O.oc(grid, rmin, x, dcf, vf, hs=hs)
        if fp32_storage:
            xn, xp = _r32(xn), _r32(xp)
        x, xphys = xn, xp
        comp.append(c)
        steps.append(nb)
        mean.append(float(xphys.mean()))
        pcg.append(its)
        if log:
            log(f"  {'fp32' if fp32_storage else 'fp64'} it {k:3d}  c {c:.10g}  bisect {nb}  pcg {its}  "
                f"{time.time() - t:.1f}s")
    E = O.moduli(xphys, mat)
    u, _, _ = O.pcg(grid, ke, E, f, mask, u0=u, tol=tol)
    return dict(compliance=np.array(comp), bisect_steps=np.array(steps, dtype=np.int32),
                mean_xphys=np.array(mean), pcg_iterations=np.array(pcg, dtype=np.int32),
                x=x.astype(np.float32), xphys=xphys.astype(np.float32), final_compliance=float(f @ u))


def make(name: str, log=print):
    case = CASES[name]
    log(f"{name}: {case}")
    ref = trajectory(case, False, log)
    drift = trajectory(case, True, log)
    rel = np.abs(drift["compliance"] - ref["compliance"]) / np.abs(ref["compliance"])
    dx = np.abs(drift["xphys"].astype(np.float64) - ref["xphys"])
    log(f"{name}: drift of FP32 storage: max rel compliance diff {rel.max():.3e} "
        f"(final {abs(drift['final_compliance'] - ref['final_compliance']) / ref['final_compliance']:.3e}), "
        f"max |dxPhys| {dx.max():.3e}, mean |dxPhys| {dx.mean():.3e}, bisection steps differ at "
        f"{int(np.sum(drift['bisect_steps'] != ref['bisect_steps']))} iterations")
    out = {k: v for k, v in ref.items()}
    out.update({"drift_" + k: v for k, v in drift.items()})
    out["grid"] = np.array(case["grid"], dtype=np.int32)
    out["rmin"], out["volfrac"], out["iters"] = case["rmin"], case["volfrac"], case["iters"]
    path = os.path.join(HERE, f"traj_{name}.npz")
    np.savez_compressed(path, **out)
    log(f"wrote {path}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=sorted(CASES), default=None)
    ap.add_argument("--threads", type=int, default=0)
    a = ap.parse_args()
    if a.threads:
        O.set_threads(a.threads)
    for name in ([a.only] if a.only else sorted(CASES)):
        make(name, log=lambda s: print(s, flush=True))


if __name__ == "__main__":
    main()
