"""``TopoDataGenerator`` with the interface of genpipeline/topology/topo_data_gen.py, driving
the batched SIMP solver.

Kept from the reference: the geometry / boundary-condition table ``GEOM_BCS`` and the
selection weights (:41-126; the class body assigns ``GEOM_WEIGHTS`` twice and the second
assignment is the one in force), the random draws and their order per sample (geometry,
grid extents for the ``grid_size``, volume fraction, force; :168-206, :226-245, with numpy's
global generator), the sample file names, the STL at threshold 0.5 with the voxel size
(100/nx, 20/ny, 20/nz) mm, and the JSON record (compliance, stress proxy 0.1 x compliance,
mass, parameters; :246-289).

Changed: instead of one solver per sample in a thread pool (:291-307), ``generate`` draws a
batch of samples and runs them together through ``BatchSIMP``. Every SIMP iteration's FEM
solves of all samples share persistent batched launches, so many small grids of uneven sizes
fill the GPU. The iteration follows ``SIMPSolverGPU.run``. Each sample gets its ``GEOM_BCS``
entry (which the reference's GPU branch drops: its ``DenseGPUSolver`` takes no boundary
conditions, :208-224) through ``bcs.generator``: the clamped faces and loads of the CPU
class, which accepts lists of faces and load directions, with the named-position and grid
loads that only the GPU class implements. The STL surface is extracted on the GPU
(``density_to_stl``).
"""
from __future__ import annotations

import json
import logging
import uuid
from pathlib import Path
from typing import List

import numpy as np

from .. import bcs as B
from .batch_simp import BatchSIMP, SimpCase
from .mesh_export import density_to_stl

log = logging.getLogger(__name__)


class TopoDataGenerator:
    GEOM_BCS = {
        "cantilever": {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2},
        "tapered": {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2},
        "ribbed": {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2},
        "lbracket": {"fixed_face": "z_min", "load_face": "x_max", "load_dof": 2},
        "bridge": {"fixed_face": ["x_min", "x_max"], "load_face": "center", "load_dof": 2},
        "arch": {"fixed_face": ["x_min", "x_max"], "load_face": "top", "load_dof": 2},
        "3dload": {"fixed_face": "x_min", "load_face": "x_max", "load_dof": [1, 2], "multi_load": True},
        "offset": {"fixed_face": "x_min", "load_face": "x_max_offset", "load_dof": 2},
        "center": {"fixed_face": "x_min", "load_face": "center_z", "load_dof": 2},
        "portal": {"fixed_face": ["y_min", "y_max"], "load_face": "top_center", "load_dof": 2},
        "spoke": {"fixed_face": "center", "load_face": "outer_ring", "load_dof": 2},
        "tower": {"fixed_face": "z_min", "load_face": "z_max", "load_dof": [1, 2]},
        "sandwich": {"fixed_face": ["z_min", "z_max"], "load_face": "center", "load_dof": 2},
        "simply": {"fixed_face": ["x_min", "x_max"], "load_face": "top", "load_dof": 2},
        "branch": {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2, "multi_load": True,
                   "load_positions": ["top", "mid", "bottom"]},
        "y_tree": {"fixed_face": "z_min", "load_face": "x_max", "load_dof": 2, "multi_load": True,
                   "load_positions": ["top", "mid_y", "mid_z"]},
        "network": {"fixed_face": ["x_min", "y_min"], "load_face": "x_max", "load_dof": 2, "multi_load": True,
                    "load_pattern": "grid"},
    }

    GEOM_WEIGHTS = {
        "bridge": 2, "arch": 2, "3dload": 2, "offset": 1, "center": 1, "cantilever": 1, "tapered": 1,
        "ribbed": 1, "lbracket": 1, "branch": 1, "y_tree": 1, "network": 1,
    }

    def __init__(self, output_dir: str = "./fem_data", n_workers: int = 2, use_gpu: bool = True, n_iters: int = 30,
                 grid_size: str = "medium", penal: float = 3.5, organic_mode: bool = True, batch_size: int = 64,
                 engine=None):
        self.output_dir = Path(output_dir)
        self.output_dir.mkdir(parents=True, exist_ok=True)
        self.n_workers = n_workers
        self.use_gpu = use_gpu
        self.n_iters = n_iters
        self.grid_size = grid_size
        self.penal = penal
        self.organic_mode = organic_mode
        self.batch_size = batch_size
        self._eng = engine
        self.written: List[dict] = []

    # ---- draws (numpy's global generator, in the reference's order) ----------------------
    def _get_grid_dims(self, geom: str):
        r = np.random.randint
        if self.grid_size == "small":
            return 16, 8, 8
        if self.grid_size == "medium":
            if geom in ("lbracket", "bridge", "arch", "center"):
                return r(16, 24), r(6, 10), r(12, 18)
            if geom in ("3dload", "offset"):
                return r(22, 32), r(8, 12), r(8, 12)
            if geom in ("branch", "y_tree", "network"):
                return r(22, 32), r(10, 16), r(10, 16)
            return r(20, 32), r(6, 10), r(6, 10)
        if geom in ("lbracket", "bridge", "arch", "center"):
            return r(24, 36), r(8, 12), r(24, 36)
        if geom in ("3dload", "offset"):
            return r(28, 40), r(8, 14), r(8, 14)
        if geom in ("branch", "y_tree", "network"):
            return r(24, 36), r(12, 18), r(12, 18)
        return r(24, 40), r(6, 12), r(6, 12)

    def _select_geometry(self):
        geoms = list(self.GEOM_BCS.keys())
        if self.organic_mode:
            w = np.array([self.GEOM_WEIGHTS.get(g, 1) for g in geoms], dtype=np.float64)
            return str(np.random.choice(geoms, p=w / w.sum()))
        return str(np.random.choice(geoms))

    def _draw(self):
        geom = self._select_geometry()
        nx, ny, nz = (int(v) for v in self._get_grid_dims(geom))
        if self.organic_mode:
            volfrac, force = np.random.uniform(0.12, 0.35), np.random.uniform(200, 5000)
        else:
            volfrac, force = np.random.uniform(0.2, 0.5), np.random.uniform(500, 2000)
        return SimpCase((nx, ny, nz), float(volfrac), float(force), dict(self.GEOM_BCS[geom]), self.penal, 1.5,
                        tag=geom)

    # ---- solve + write ---------------------------------------------------------------------
    def _solve(self, cases: List[SimpCase]) -> List[SimpCase]:
        if self.use_gpu:
            return BatchSIMP(cases, engine=self._eng, bc_fn=B.generator).run(self.n_iters)
        from .simp_solver import SIMPSolver

        for c in cases:
            s = SIMPSolver(nx=c.grid[0], ny=c.grid[1], nz=c.grid[2], penal=c.penal, rmin=c.rmin,
                           boundary_conditions=c.bcs)
            c.density = s.run(volfrac=c.volfrac, n_iters=self.n_iters, force_mag=c.force_mag)
            c.last_compliance = s.last_compliance
        return cases

    def _write(self, c: SimpCase) -> dict:
        geom = c.tag
        nx, ny, nz = c.grid
        stem = f"{geom[:4]}_v{int(c.volfrac * 100)}_f{int(c.force_mag)}_{nx}x{ny}x{nz}_{str(uuid.uuid4())[:8]}"
        stl_path = self.output_dir / f"{stem}_mesh.stl"
        json_path = self.output_dir / f"{stem}_fem_results.json"
        if c.failed or c.density is None:
            raise ValueError(f"SIMP failed for {geom}")
        if density_to_stl(c.density, str(stl_path), threshold=0.5,
                          voxel_size_mm=(100.0 / nx, 20.0 / ny, 20.0 / nz)) is None:
            raise ValueError(f"Empty design for {geom}")
        compliance = c.last_compliance
        total_vol = 100.0 * 20.0 * 100.0 if geom in ("lbracket", "bridge", "arch") else 100.0 * 20.0 * 20.0
        results = {
            "stress_max": float(compliance * 0.1),
            "compliance": float(compliance),
            "mass": float(c.density.mean() * total_vol * 1.05e-6),
            "parameters": {"geometry": geom, "volfrac": float(c.volfrac), "force_n": float(c.force_mag),
                           "nx": int(nx), "ny": int(ny), "nz": int(nz), "penal": self.penal},
        }
        with open(json_path, "w") as fh:
            json.dump(results, fh, indent=2)
        rec = {"stl": str(stl_path), "json": str(json_path), **results}
        self.written.append(rec)
        return rec

    def _run_batch(self, cases: List[SimpCase], first: int, n_samples: int) -> int:
        ok = 0
        for k, c in enumerate(self._solve(cases)):
            try:
                rec = self._write(c)
                ok += 1
                log.info(f"[{first + k + 1}/{n_samples}] Generated {c.tag}: {Path(rec['stl']).name}")
            except Exception as e:  # the reference logs a failed sample and goes on (:301-307)
                log.error(f"Sample generation failed: {e}")
        return ok

    def generate_single(self, i, n_samples):
        c = self._draw()
        self._solve([c])
        rec = self._write(c)
        log.info(f"[{i + 1}/{n_samples}] Generated {c.tag}: {Path(rec['stl']).name}")

    def generate(self, n_samples: int = 100) -> int:
        """Draws and solves the samples in batches of ``batch_size``; returns how many were
        written."""
        ok = 0
        for first in range(0, n_samples, self.batch_size):
            cases = [self._draw() for _ in range(min(self.batch_size, n_samples - first))]
            ok += self._run_batch(cases, first, n_samples)
        return ok

    def generate_scaled(self, n_samples: int = 1000, batch_size: int = 100) -> int:
        ok = 0
        for first in range(0, n_samples, batch_size):
            cases = [self._draw() for _ in range(min(batch_size, n_samples - first))]
            ok += self._run_batch(cases, first, n_samples)
            log.info(f"Progress: {min(first + batch_size, n_samples)}/{n_samples} samples generated")
        return ok
