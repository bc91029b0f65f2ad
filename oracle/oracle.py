"""ctypes front end of the FP64 oracle (``oracle/simp_oracle.c``). Test infrastructure only.

Every function mirrors one step of the reference CPU solver
``genpipeline/topology/simp_solver.py`` (see the C file's header for the line map) and
works on float64 numpy arrays in the reference's layout (element e = i*ny*nz + j*nz + k,
DOF 3n + c).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

_D = C.POINTER(C.c_double)
_U8 = C.POINTER(C.c_uint8)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.orc_num_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_ke_quadrature.argtypes = [C.c_double, C.c_double, _D]
        L.orc_moduli.argtypes = [C.c_int64, _D, C.c_int, C.c_double, C.c_double, C.c_double,
                                 C.c_double, _D]
        L.orc_apply.argtypes = [C.c_int] * 3 + [_D, _D, _D, _U8, _D]
        L.orc_diag.argtypes = [C.c_int] * 3 + [_D, _D, _U8, _D]
        L.orc_element_energy.argtypes = [C.c_int] * 3 + [_D, _D, _D, C.c_int] + [C.c_double] * 4 + [_D, _D]
        L.orc_element_energy.restype = C.c_double
        L.orc_filter_hs.argtypes = [C.c_int] * 3 + [C.c_double, _D]
        L.orc_filter.argtypes = [C.c_int] * 3 + [C.c_double, _D, _D, C.c_int, _D]
        L.orc_oc.argtypes = ([C.c_int] * 3 + [C.c_double, _D, _D, _D, _U8] + [C.c_double] * 4
                             + [C.c_int] + [C.c_double] * 3 + [_D, _D])
        L.orc_oc.restype = C.c_int
        L.orc_pcg.argtypes = [C.c_int] * 3 + [_D, _D, _D, _U8, _D, C.c_double, C.c_int, _D]
        L.orc_pcg.restype = C.c_int
        L.orc_simp_step.argtypes = ([C.c_int] * 3 + [_D, C.c_int] + [C.c_double] * 5
                                    + [_D, _D, _U8, _U8, C.c_double, _D, _D, _D, C.c_double,
                                       C.c_int, _D, _D])
        L.orc_simp_step.restype = C.c_int
        L.orc_simp_run.argtypes = ([C.c_int] * 3 + [_D, C.c_int] + [C.c_double] * 5
                                   + [_D, _U8, _U8, C.c_double, C.c_int, C.c_double, C.c_int,
                                      _D, _D, _D, _D])
        L.orc_simp_run.restype = C.c_long
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_D)


def _u8(a):
    return None if a is None else a.ctypes.data_as(_U8)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _mask(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.uint8)


LAWS = {"ref": 0, "modified": 1}


class Material:
    """Stiffness law: ``ref`` = e0*max(x,xmin)^p (simp_solver.py:182-185); ``modified`` =
    emin + x^p (e0-emin)."""

    def __init__(self, law="ref", penal=3.0, e0=1.0, emin=1e-9, xmin=1e-3):
        self.law, self.penal, self.e0, self.emin, self.xmin = law, penal, e0, emin, xmin

    def args(self):
        return (LAWS[self.law], self.penal, self.e0, self.emin, self.xmin)


def num_threads() -> int:
    return lib().orc_num_threads()


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def ke_quadrature(nu=0.3, e0=1.0) -> np.ndarray:
    ke = np.zeros(576)
    lib().orc_ke_quadrature(nu, e0, _d(ke))
    return ke.reshape(24, 24)


def moduli(x, mat: Material) -> np.ndarray:
    x = _f64(x)
    E = np.empty_like(x)
    lib().orc_moduli(x.size, _d(x), *mat.args(), _d(E))
    return E


def apply(grid, ke, E, p, fixed=None) -> np.ndarray:
    nx, ny, nz = grid
    ke, E, p, fixed = _f64(ke), _f64(E), _f64(p), _mask(fixed)
    y = np.empty_like(p)
    lib().orc_apply(nx, ny, nz, _d(ke), _d(E), _d(p), _u8(fixed), _d(y))
    return y


def diag(grid, ke, E, fixed=None) -> np.ndarray:
    nx, ny, nz = grid
    ke, E, fixed = _f64(ke), _f64(E), _mask(fixed)
    d = np.empty(3 * (nx + 1) * (ny + 1) * (nz + 1))
    lib().orc_diag(nx, ny, nz, _d(ke), _d(E), _u8(fixed), _d(d))
    return d


def element_energy(grid, ke, x, u, mat: Material):
    """Returns (ce, dc, u^T K u)."""
    nx, ny, nz = grid
    ke, x, u = _f64(ke), _f64(x), _f64(u)
    ce = np.empty(nx * ny * nz)
    dc = np.empty(nx * ny * nz)
    tot = lib().orc_element_energy(nx, ny, nz, _d(ke), _d(x), _d(u), *mat.args(), _d(ce), _d(dc))
    return ce, dc, tot


def filter_hs(grid, rmin) -> np.ndarray:
    nx, ny, nz = grid
    hs = np.empty(nx * ny * nz)
    lib().orc_filter_hs(nx, ny, nz, float(rmin), _d(hs))
    return hs


def density_filter(grid, rmin, v, hs=None, transpose=False) -> np.ndarray:
    nx, ny, nz = grid
    hs = filter_hs(grid, rmin) if hs is None else _f64(hs)
    v = _f64(v)
    out = np.empty_like(v)
    lib().orc_filter(nx, ny, nz, float(rmin), _d(hs), _d(v), int(bool(transpose)), _d(out))
    return out


OC_CPU = dict(move=0.2, l1=0.0, l2=1e9, max_bisect=50, tol=1e-4, tol_eps=1e-12, sqrt_floor=1e-12)
OC_GPU = dict(move=0.2, l1=0.0, l2=-1.0, max_bisect=30, tol=1e-5, tol_eps=1e-15, sqrt_floor=1e-15)


def oc(grid, rmin, x, dc, volfrac, preserved=None, hs=None, variant=OC_CPU):
    """Returns (xnew, xphys_new, bisection steps)."""
    nx, ny, nz = grid
    hs = filter_hs(grid, rmin) if hs is None else _f64(hs)
    x, dc, pres = _f64(x), _f64(dc), _mask(preserved)
    xn = np.empty_like(x)
    xp = np.empty_like(x)
    v = variant
    it = lib().orc_oc(nx, ny, nz, float(rmin), _d(hs), _d(x), _d(dc), _u8(pres), float(volfrac),
                      v["move"], v["l1"], v["l2"], v["max_bisect"], v["tol"], v["tol_eps"],
                      v["sqrt_floor"], _d(xn), _d(xp))
    return xn, xp, it


def pcg(grid, ke, E, f, fixed=None, u0=None, tol=1e-12, max_iter=100000):
    """Returns (u, iterations, relres)."""
    nx, ny, nz = grid
    ke, E, f, fixed = _f64(ke), _f64(E), _f64(f), _mask(fixed)
    u = np.zeros_like(f) if u0 is None else _f64(u0).copy()
    rel = C.c_double(0.0)
    it = lib().orc_pcg(nx, ny, nz, _d(ke), _d(E), _d(f), _u8(fixed), _d(u), float(tol),
                       int(max_iter), C.byref(rel))
    return u, it, rel.value


class SimpState:
    """Holds the arrays of an oracle SIMP run so that it can be stepped one OC iteration
    at a time (the unit ``bench.py`` times)."""

    def __init__(self, grid, ke, mat: Material, rmin, f, fixed, volfrac, preserved=None,
                 tol=1e-8, max_iter=100000):
        self.grid, self.ke, self.mat, self.rmin = tuple(grid), _f64(ke), mat, float(rmin)
        nx, ny, nz = grid
        ne = nx * ny * nz
        self.f, self.fixed, self.pres = _f64(f), _mask(fixed), _mask(preserved)
        self.volfrac, self.tol, self.max_iter = float(volfrac), float(tol), int(max_iter)
        self.hs = filter_hs(grid, rmin)
        self.x = np.full(ne, self.volfrac)
        if self.pres is not None:
            self.x[self.pres.astype(bool)] = 1.0
        self.xphys = self.x.copy()
        self.u = np.zeros_like(self.f)
        self.compliance = float("nan")
        self.last_iters = 0

    def step(self):
        nx, ny, nz = self.grid
        c = C.c_double(0.0)
        dcf = np.empty(nx * ny * nz)
        self.last_iters = lib().orc_simp_step(
            nx, ny, nz, _d(self.ke), *self.mat.args(), self.rmin, _d(self.hs), _d(self.f),
            _u8(self.fixed), _u8(self.pres), self.volfrac, _d(self.x), _d(self.xphys),
            _d(self.u), self.tol, self.max_iter, C.byref(c), _d(dcf))
        self.compliance = c.value
        self.dc = dcf
        return self.last_iters


def simp_run(grid, ke, mat: Material, rmin, f, fixed, volfrac, n_iters, preserved=None,
             tol=1e-10, max_iter=100000):
    """SIMPSolver.run: returns (x, xphys, u, compliance, total PCG iterations)."""
    nx, ny, nz = grid
    ne = nx * ny * nz
    ke, f, fixed, pres = _f64(ke), _f64(f), _mask(fixed), _mask(preserved)
    x = np.empty(ne)
    xp = np.empty(ne)
    u = np.empty_like(f)
    c = C.c_double(0.0)
    tot = lib().orc_simp_run(nx, ny, nz, _d(ke), *mat.args(), float(rmin), _d(f), _u8(fixed),
                             _u8(pres), float(volfrac), int(n_iters), float(tol), int(max_iter),
                             _d(x), _d(xp), _d(u), C.byref(c))
    return x, xp, u, c.value, tot


def simp_gpu_run(grid, rmin, penal, f, fixed, volfrac, n_iters, preserved=None, x_init=None,
                 schedule=None, direct_below=50000, exact_tol=1e-12, compliance_tol=1e-6,
                 compliance_max_iter=2000, fp32_storage=False):
    """``SIMPSolverGPU.run`` (genpipeline/topology/simp_solver_gpu.py:71-136) in FP64.

    - x_init rescaled to the volume fraction and clamped to [1e-3, 1] (:80-84);
      preserved elements set to 1 (:88-89);
    - per iteration: the sensitivity solve warm-started from the last displacement with the
      tolerance schedule (:92-99, ``schedule(i) -> (tol, max_iter)``), dc of the floored law
      max(x, 1e-3)^penal (:753-794), the filter chain rule (:796-799), the GPU OC variant
      (:801-841), then a cold compliance solve at the new design whose displacement
      warm-starts the next iteration (:111, :747-751, ``_u_prev`` at :586-607);
    - the early stop after three relative compliance changes below 1% (:113-125).
    ``_solve`` solves directly (SuperLU) whenever the grid has fewer than 50,000 DOFs
    (:581-588), whatever the tolerance: those solves run here to ``exact_tol``.
    ``fp32_storage`` (True, or "keep_start" to leave the initial design unrounded) rounds dc,
    the filtered dc, x and xPhys to float32 where a single-precision implementation stores
    them: the drift that storage alone causes.
    Returns dict(xphys, history, last_compliance, iterations)."""
    nx, ny, nz = grid
    ne = nx * ny * nz
    nd = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    mat = Material("ref", penal)
    ke = ke_quadrature()
    hs = filter_hs(grid, rmin)
    f = _f64(f)
    pres = None if preserved is None else np.asarray(preserved).reshape(-1).astype(bool)
    if x_init is not None:
        x = _f64(np.asarray(x_init).reshape(-1))
        x = np.clip(x * (volfrac / max(x.mean(), 1e-6)), 1e-3, 1.0)
    else:
        x = np.full(ne, float(volfrac))
    if pres is not None:
        x[pres] = 1.0
    xphys = x.copy()
    direct = nd < direct_below
    if schedule is None:
        def schedule(i):
            return (1e-4, 200) if i < 3 else (1e-5, 400) if i < 8 else (1e-6, 800)

    def solve(u0, tol, max_iter):
        if direct:
            tol, max_iter = exact_tol, 1000000
        u, _, _ = pcg(grid, ke, moduli(xphys, mat), f, fixed, u0=u0, tol=tol, max_iter=max_iter)
        return u

    u_prev = None
    prev, changes, history = float("inf"), [], []
    curr = float("nan")
    it = 0
    pmask = None if pres is None else pres.astype(np.uint8)
    r32 = (lambda a: a.astype(np.float32).astype(np.float64)) if fp32_storage else (lambda a: a)
    hs = r32(hs)
    if fp32_storage != "keep_start":  # "keep_start": the initial design stays exact
        x, xphys = r32(x), r32(xphys)
    for i in range(n_iters):
        tol, max_iter = schedule(i)
        u = solve(u_prev, tol, max_iter)
        _, dc, _ = element_energy(grid, ke, xphys, u, mat)
        dcf = r32(density_filter(grid, rmin, r32(dc), hs=hs, transpose=True))
        x, xphys, _ = oc(grid, rmin, x, dcf, volfrac, preserved=pmask, hs=hs, variant=OC_GPU)
        x, xphys = r32(x), r32(xphys)
        uc = solve(None, compliance_tol, compliance_max_iter)
        u_prev = uc
        curr = float(f @ uc)
        history.append(curr)
        it = i + 1
        if prev != float("inf"):
            changes.append(abs(prev - curr) / (prev + 1e-10))
        if len(changes) >= 3 and all(c < 0.01 for c in changes[-3:]):
            break
        prev = curr
    return dict(xphys=xphys, history=np.array(history), last_compliance=curr, iterations=it)
