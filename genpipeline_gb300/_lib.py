"""ctypes binding of ``libgbsimp.so`` (the C ABI declared in ``include/gbsimp.h``).

There is no fallback: if the library is missing or does not load, every entry point
raises. ``build.build()`` (or ``__graft_entry__.build()``) compiles it in-tree.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

GBS_OK = 0
GBS_EINVAL = 1
GBS_ENOMEM = 2
GBS_ENOTCONV = 3
GBS_EBREAKDOWN = 4
GBS_ETIMEOUT = 5
GBS_ECUDA = 6
GBS_ENONFINITE = 7

STATUS_NAMES = {
    GBS_OK: "ok",
    GBS_EINVAL: "invalid argument",
    GBS_ENOMEM: "out of memory",
    GBS_ENOTCONV: "not converged",
    GBS_EBREAKDOWN: "breakdown",
    GBS_ETIMEOUT: "timeout",
    GBS_ECUDA: "cuda error",
    GBS_ENONFINITE: "non-finite",
}


class GbsimpError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gbsimp error {code} ({STATUS_NAMES.get(code, '?')}): {msg}")
        self.code = code


class Law(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("penal", C.c_double),
                ("e0", C.c_double), ("emin", C.c_double), ("xmin", C.c_double)]


class OcParams(C.Structure):
    _fields_ = [("move", C.c_double), ("l1", C.c_double), ("l2", C.c_double), ("tol", C.c_double),
                ("tol_eps", C.c_double), ("sqrt_floor", C.c_double), ("volfrac", C.c_double),
                ("max_bisect", C.c_int32), ("reserved", C.c_int32)]


class SolveOpts(C.Structure):
    _fields_ = [("rtol", C.c_double), ("inner_rtol", C.c_double), ("max_iter", C.c_int32),
                ("max_outer", C.c_int32), ("check_every", C.c_int32), ("fused", C.c_int32),
                ("profile", C.c_int32), ("batch_share", C.c_int32), ("batch_group", C.c_int32),
                ("residual_fp64", C.c_int32)]


class SolveStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int32), ("outer", C.c_int32),
                ("inner_active", C.c_int32), ("relres", C.c_double), ("seconds", C.c_double),
                ("apply_seconds", C.c_double), ("apply_launches", C.c_int32), ("inner_iters", C.c_int32)]

    def as_dict(self):
        return {"status": int(self.status), "status_name": STATUS_NAMES.get(int(self.status), "?"),
                "iterations": int(self.iterations), "outer": int(self.outer),
                "relres": float(self.relres), "seconds": float(self.seconds),
                "apply_seconds": float(self.apply_seconds), "apply_launches": int(self.apply_launches)}


class BatchItem(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("state", C.c_int32),
                ("x", C.c_void_p), ("f", C.c_void_p), ("node_mask", C.c_void_p), ("u", C.c_void_p),
                ("ws", C.c_void_p), ("ws_bytes", C.c_size_t), ("stats", SolveStats)]


class SimpOpts(C.Structure):
    _fields_ = [("volfrac", C.c_double), ("rmin", C.c_double), ("n_iters", C.c_int32), ("early_stop", C.c_int32),
                ("oc", OcParams), ("solve", SolveOpts)]


_P = C.c_void_p
_I = C.c_int
_I64 = C.c_int64
_D = C.c_double
_SZ = C.c_size_t

# name -> (restype, argtypes); the list mirrors include/gbsimp.h one to one.
SIGNATURES = {
    "gbsimp_abi_version": (_I, []),
    "gbsimp_launch_count": (C.c_uint64, []),
    "gbsimp_last_error": (C.c_char_p, []),
    "gbsimp_create": (_I, [C.POINTER(_P)]),
    "gbsimp_destroy": (_I, [_P]),
    "gbsimp_ke_quadrature": (_I, [_D, _D, C.POINTER(_D)]),
    "gbsimp_set_ke": (_I, [_P, C.POINTER(_D)]),
    "gbsimp_get_ke": (_I, [_P, C.POINTER(_D)]),
    "gbsimp_apply_f32": (_I, [_P, _I, _I, _I, C.POINTER(Law), _P, _P, _P, _P, _P]),
    "gbsimp_apply_path": (_I, [_P, _I]),
    "gbsimp_apply_f64": (_I, [_P, _I, _I, _I, C.POINTER(Law), _P, _P, _P, _P, _P]),
    "gbsimp_apply_edof_f32": (_I, [_P, _I64, _I64, _P, _I, C.POINTER(Law), _P, _P, _P, _P]),
    "gbsimp_sensitivity_ws_bytes": (_SZ, [_I, _I, _I]),
    "gbsimp_sensitivity": (_I, [_P, _I, _I, _I, C.POINTER(Law), _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "gbsimp_sensitivity_edof_f32": (_I, [_P, _I64, _I64, _P, _I, C.POINTER(Law), _P, _P, _P, _P]),
    "gbsimp_filter_hs": (_I, [_P, _I, _I, _I, _D, _P, _P]),
    "gbsimp_filter": (_I, [_P, _I, _I, _I, _D, _P, _P, _P, _I, _P]),
    "gbsimp_oc_ws_bytes": (_SZ, [_I, _I, _I]),
    "gbsimp_oc_prepare": (_I, [_P, _I, _I, _I, _D, _P, _P, _SZ, _P]),
    "gbsimp_oc": (_I, [_P, _I, _I, _I, _D, C.POINTER(OcParams), _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "gbsimp_oc_noalloc": (_I, [_P, _I, _I, _I, _D, C.POINTER(OcParams), _P, _P, _P, _P, _P, _P]),
    "gbsimp_oc_result": (_I, [_P, _P, C.POINTER(_D), C.POINTER(_I), _P]),
    "gbsimp_pcg_ws_bytes": (_SZ, [_I, _I, _I]),
    "gbsimp_pcg_f32": (_I, [_P, _I, _I, _I, C.POINTER(Law), _P, _P, _P, _P, C.POINTER(SolveOpts),
                            C.POINTER(SolveStats), _P, _SZ, _P]),
    "gbsimp_time_pcg_apply_ws_bytes": (_SZ, [_I, _I, _I]),
    "gbsimp_time_pcg_apply": (_I, [_P, _I, _I, _I, C.POINTER(Law), _P, _P, _I, _P, _SZ, C.POINTER(_D), _P]),
    "gbsimp_solve_ws_bytes": (_SZ, [_I, _I, _I]),
    "gbsimp_solve": (_I, [_P, _I, _I, _I, C.POINTER(Law), _P, _P, _P, _P, C.POINTER(SolveOpts),
                          C.POINTER(SolveStats), _P, _SZ, _P]),
    "gbsimp_batch_round": (_I, [_P, C.POINTER(BatchItem), _I, C.POINTER(Law), C.POINTER(SolveOpts), _P]),
    "gbsimp_batch_solve": (_I, [_P, C.POINTER(BatchItem), _I, C.POINTER(Law), C.POINTER(SolveOpts), _P]),
    "gbsimp_queue_create": (_I, [_P, C.POINTER(Law), C.POINTER(SolveOpts), C.POINTER(_P)]),
    "gbsimp_queue_destroy": (_I, [_P]),
    "gbsimp_queue_submit": (_I, [_P, C.POINTER(BatchItem)]),
    "gbsimp_queue_poll": (_I, [_P, C.POINTER(C.POINTER(BatchItem)), _I, C.POINTER(C.c_int), _P]),
    "gbsimp_queue_size": (_I, [_P]),
    "gbsimp_simp_run_ws_bytes": (_SZ, [_I, _I, _I]),
    "gbsimp_simp_run": (_I, [_P, _I, _I, _I, C.POINTER(Law), C.POINTER(SimpOpts), _P, _P, _P, _P, _P, _P,
                             C.POINTER(_D), C.POINTER(C.c_int32), C.POINTER(SolveStats), _P, _SZ, _P]),
    "gbsimp_pcg_csr_ws_bytes": (_SZ, [_I64]),
    "gbsimp_pcg_csr_f32": (_I, [_P, _I64, _P, _P, _P, _P, _P, _P, _P, _I64, C.POINTER(SolveOpts),
                                C.POINTER(SolveStats), _P, _SZ, _P]),
    "gbsimp_dot_f64": (_I, [_P, _I64, _P, _P, _P, _P, _SZ, _P]),
    "gbsimp_warm_start": (_I, [_P, _I64, _P, _P, _D, _P]),
    "gbsimp_voxel_prep_ws_bytes": (_SZ, [_I, _I, _I, _I, _I, _I, _I]),
    "gbsimp_voxel_prep": (_I, [_P, _I, _I, _I, _I, _P, _I, _I, _I, _P, _D, _D, _P, _SZ, _P]),
    "gbsimp_barrier_selftest_ws_bytes": (_SZ, []),
    "gbsimp_barrier_selftest": (_I, [_P, _I, _D, C.POINTER(C.c_int), _P, _SZ, _P]),
    "gbsimp_marching_cubes_ws_bytes": (_SZ, [_I, _I, _I]),
    "gbsimp_marching_cubes_table": (_I, [_P, _P, _P, _P]),
    "gbsimp_marching_cubes": (_I, [_P, _I, _I, _I, _P, _D, _D, _D, _D, _P, _I64, C.POINTER(C.c_int64), _P, _SZ,
                                   _P]),
}

_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads the library (building it first when it is missing or stale and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing and not _build.up_to_date():
            try:
                _build.build()
            except Exception as exc:  # pragma: no cover - surfaced below
                if not os.path.exists(path):
                    raise GbsimpError(GBS_ECUDA, f"libgbsimp.so is missing and the build failed: {exc}")
        if not os.path.exists(path):
            raise GbsimpError(GBS_ECUDA, f"libgbsimp.so not found at {path}; run genpipeline_gb300.build")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(code: int) -> int:
    if code != GBS_OK:
        msg = load().gbsimp_last_error()
        raise GbsimpError(code, msg.decode() if msg else "")
    return code


def make_law(kind="ref", penal=3.0, e0=1.0, emin=1e-9, xmin=1e-3) -> Law:
    k = {"ref": 0, "modified": 1}[kind] if isinstance(kind, str) else int(kind)
    return Law(k, 0, float(penal), float(e0), float(emin), float(xmin))


OC_CPU = dict(move=0.2, l1=0.0, l2=1e9, tol=1e-4, tol_eps=1e-12, sqrt_floor=1e-12, max_bisect=50)
OC_GPU = dict(move=0.2, l1=0.0, l2=-1.0, tol=1e-5, tol_eps=1e-15, sqrt_floor=1e-15, max_bisect=30)


def make_oc(volfrac, variant=None) -> OcParams:
    v = dict(OC_CPU if variant is None else variant)
    return OcParams(v["move"], v["l1"], v["l2"], v["tol"], v["tol_eps"], v["sqrt_floor"],
                    float(volfrac), int(v["max_bisect"]), 0)
