"""Many SIMP problems of uneven sizes advanced in lockstep, their FEM solves batched.

Each problem follows ``SIMPSolverGPU.run`` (topology/simp_solver_gpu.py:71-136): per
iteration a warm-started sensitivity solve with the tolerance schedule (1e-4 / 200 PCG
iterations for iterations 0-2, 1e-5 / 400 for 3-7, 1e-6 / 800 after; grids below 50,000
DOFs to 1e-10, as the reference solves those directly), the floored law
``max(x, 1e-3)^penal``, the filtered sensitivity, the GPU OC variant, then a fresh compliance
solve (1e-6 / 2000) whose displacement warm-starts the next iteration, and the early stop
after three changes of compliance below 1%. The solves of all problems still running go
through ``BatchFEM`` rounds together (one persistent launch per round, up to 24 designs per
launch, each on its own share of the SMs). The sensitivity, filter and OC steps are launched
per problem on the same stream. ``bc_fn(nx, ny, nz, bcs, force)`` gives each problem's load
and clamped DOFs (default: ``SIMPSolverGPU._get_bcs``).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import torch

from .. import _lib as L
from .. import bcs as B
from ..batch import BatchFEM, FEMDesign
from ..engine import Engine, get_engine, n_dof, n_elem


# SIMPSolverGPU._solve factorises K directly below this many DOFs, ignoring the tolerance it
# is given (simp_solver_gpu.py:581-588); such solves run to DIRECT_RTOL here.
DIRECT_BELOW = 50000
DIRECT_RTOL = 1e-10


def reference_schedule(i: int):
    """(tol, max_iter) of the sensitivity solve at iteration i (simp_solver_gpu.py:92-99)."""
    if i < 3:
        return 1e-4, 200
    if i < 8:
        return 1e-5, 400
    return 1e-6, 800


@dataclass
class SimpCase:
    grid: tuple
    volfrac: float
    force_mag: float = 1.0
    bcs: Optional[dict] = None
    penal: float = 3.0
    rmin: float = 1.5
    tag: object = None
    # results
    density: Optional[np.ndarray] = field(default=None, repr=False)
    last_compliance: float = float("nan")
    history: List[float] = field(default_factory=list)
    iterations: int = 0
    failed: bool = False


class BatchSIMP:
    def __init__(self, cases: List[SimpCase], engine: Optional[Engine] = None, schedule=reference_schedule,
                 compliance_tol: float = 1e-6, compliance_max_iter: int = 2000, bc_fn=B.reference_gpu):
        self.eng = engine or get_engine()
        self.cases = cases
        self.schedule = schedule
        self.compliance_tol = compliance_tol
        self.compliance_max_iter = compliance_max_iter
        dev = self.eng.device
        self._st = []
        for k, c in enumerate(cases):
            nx, ny, nz = c.grid
            f, fixed = bc_fn(nx, ny, nz, c.bcs, c.force_mag)
            fem = FEMDesign(c.grid, np.zeros(n_elem(c.grid), np.float32), f, fixed, tag=k)
            BatchFEM(self.eng).upload(fem)
            x = torch.full((n_elem(c.grid),), float(c.volfrac), device=dev, dtype=torch.float32)
            s = {"fem": fem, "x": x, "xphys": x.clone(), "u": None, "prev": float("inf"), "changes": [],
                 "hs": self.eng.filter_hs(c.grid, c.rmin), "oc_key": f"bsimp:{id(self)}:{k}",
                 "law": L.make_law("ref", c.penal), "done": False, "curr": float("nan")}
            self.eng.oc_prepare(c.grid, c.rmin, None, key=s["oc_key"])
            self._st.append(s)

    def _solve(self, idx: List[int], tol: float, max_iter: int, warm: bool):
        """Batched solves of the given problems; returns {k: FEMDesign}. Problems below
        DIRECT_BELOW DOFs are solved to DIRECT_RTOL (the reference solves them directly)."""
        groups = {}
        for k in idx:
            direct = n_dof(self.cases[k].grid) < DIRECT_BELOW
            groups.setdefault((self.cases[k].penal, direct), []).append(k)
        out = {}
        for (penal, direct), ks in groups.items():
            rt, mi = (DIRECT_RTOL, 1000000) if direct else (tol, max_iter)
            bf = BatchFEM(self.eng, L.make_law("ref", penal), rtol=rt, max_iter=mi)
            for k in ks:
                s = self._st[k]
                d = s["fem"]
                d.dx = s["xphys"]
                if warm and s["u"] is not None:
                    d.du = s["u"].clone()
                else:
                    d.du = torch.zeros(n_dof(self.cases[k].grid), dtype=torch.float64, device=self.eng.device)
                bf.add(d)
            for d in bf.solve_all([]):
                out[d.tag] = d
        return out

    def run(self, n_iters: int) -> List[SimpCase]:
        eng = self.eng
        for i in range(n_iters):
            active = [k for k, s in enumerate(self._st) if not s["done"]]
            if not active:
                break
            tol, max_iter = self.schedule(i)
            sol = self._solve(active, tol, max_iter, warm=True)
            for k in active:
                c, s = self.cases[k], self._st[k]
                d = sol[k]
                if d.stats["status"] not in (L.GBS_OK, L.GBS_ENOTCONV):
                    d.du.fill_(float("nan"))
                dc = eng.sensitivity(c.grid, s["law"], s["xphys"], d.du)
                if torch.isnan(dc).any():
                    s["done"], c.failed = True, True
                    continue
                dcf = eng.filter(c.grid, c.rmin, dc, hs=s["hs"], transpose=True)
                s["x"], s["xphys"] = eng.oc(c.grid, c.rmin, c.volfrac, s["x"], dcf, None, L.OC_GPU,
                                            key=s["oc_key"], prepared=True)
            active = [k for k in active if not self._st[k]["done"]]
            comp = self._solve(active, self.compliance_tol, self.compliance_max_iter, warm=False)
            for k in active:
                c, s = self.cases[k], self._st[k]
                d = comp[k]
                if d.stats["status"] not in (L.GBS_OK, L.GBS_ENOTCONV):
                    d.du.fill_(float("nan"))
                s["u"] = d.du.clone()  # the compliance solve's u warm-starts the next iteration
                curr = float(torch.dot(d.df, d.du).item())
                s["curr"] = curr
                c.history.append(curr)
                c.iterations = i + 1
                if s["prev"] != float("inf"):
                    s["changes"].append(abs(s["prev"] - curr) / (s["prev"] + 1e-10))
                if len(s["changes"]) >= 3 and all(v < 0.01 for v in s["changes"][-3:]):
                    s["done"] = True
                s["prev"] = curr
        for c, s in zip(self.cases, self._st):
            c.last_compliance = s["curr"]
            c.density = s["xphys"].reshape(c.grid).cpu().numpy()
        return self.cases
