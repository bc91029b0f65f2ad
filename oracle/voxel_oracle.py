"""FP64 numpy restatement of the evaluator's steps around the FEM solve. Test infrastructure
only: the tests, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` use it as the
checker; the package never imports it.

* ``voxel_prep``   -- ``scipy.ndimage.zoom(v, z, order=1)`` followed by ``smooth_voxels``
  (``genpipeline/fem/voxel_fem.py:457-462``, ``genpipeline/pipeline_utils.py:55-76``),
  written as one banded matrix per axis: linear resampling (output o reads input coordinate
  o (n_in - 1) / (n_out - 1)), then a normalised Gaussian of radius int(4 sigma + 0.5) with
  the mirror boundary d c b a | a b c d | d c b a, then the logistic. Pinned against the
  reference's own output in ``tests/golden/voxel.npz``.
* ``fem_proxies``  -- the outputs of ``GPUVoxelFEM.solve`` from a displacement
  (``genpipeline/fem/gpu_fem_solver.py:98-133``) and the mass of
  ``VoxelFEMEvaluator.evaluate`` (``voxel_fem.py:477-490``).
"""
from __future__ import annotations

import numpy as np

FEM_SENTINEL = 1e6  # pipeline_utils.py:20


def _reflect(j: int, n: int) -> int:
    period = 2 * n
    j %= period
    return j if j < n else period - 1 - j


def zoom_matrix(n_in: int, n_out: int) -> np.ndarray:
    z = np.zeros((n_out, n_in))
    s = (n_in - 1) / (n_out - 1) if n_out > 1 else 0.0
    for o in range(n_out):
        p = o * s
        i0 = int(np.floor(p))
        w = p - i0
        z[o, i0] += 1.0 - w
        if i0 + 1 < n_in:
            z[o, i0 + 1] += w
    return z


def gauss_matrix(n: int, sigma: float) -> np.ndarray:
    r = int(4.0 * sigma + 0.5) if sigma > 0 else 0
    t = np.arange(-r, r + 1)
    k = np.exp(-0.5 / (sigma * sigma) * t.astype(np.float64) ** 2) if r > 0 else np.ones(1)
    k = k / k.sum()
    g = np.zeros((n, n))
    for o in range(n):
        for ti, kt in zip(t, k):
            g[o, _reflect(o + int(ti), n)] += kt
    return g


def out_shape(shape, zoom: float):
    """scipy's output shape: round(n * zoom) per axis (Python rounding)."""
    return tuple(int(round(n * zoom)) for n in shape)


def voxel_prep(vol: np.ndarray, shape_out, sigma: float = 0.5, sharpness: float = 15.0) -> np.ndarray:
    v = np.asarray(vol, dtype=np.float64)
    for axis in range(3):
        n_in, n_out = v.shape[axis], shape_out[axis]
        a = gauss_matrix(n_out, sigma) @ zoom_matrix(n_in, n_out)
        v = np.moveaxis(np.tensordot(a, v, axes=([1], [axis])), 0, axis)
    return 1.0 / (1.0 + np.exp(-sharpness * (v - 0.5)))


def fem_proxies(voxels: np.ndarray, u: np.ndarray, f: np.ndarray, bbox=None) -> dict:
    """GPUVoxelFEM.solve's outputs for displacement u under load f, plus the evaluator's mass."""
    vox = np.asarray(voxels, dtype=np.float64)
    compliance = float(np.dot(u, f))
    disp_abs = float(np.linalg.norm(np.asarray(u).reshape(-1, 3), axis=1).max())
    disp_max_mm = float(np.clip(disp_abs * 0.001 * 1e3, 0, 1e4))
    n_solid = int((vox.reshape(-1) > 0.5).sum())
    if n_solid < 50 or not np.isfinite(compliance) or compliance < 1.0:
        res = {"stress_max": 1e4, "displacement_max": 1e3, "compliance": 1e6}
    else:
        res = {"stress_max": float(np.clip(compliance / max(n_solid, 1) * 10.0, 0, 1e4)),
               "displacement_max": disp_max_mm, "compliance": float(np.clip(compliance, 0, 1e8))}
    solid_frac = float((vox > 0.5).mean())
    if bbox:
        vol_mm3 = ((bbox["x"][1] - bbox["x"][0]) * (bbox["y"][1] - bbox["y"][0])
                   * (bbox["z"][1] - bbox["z"][0])) * solid_frac
    else:
        vol_mm3 = vox.size * solid_frac
    res["mass"] = vol_mm3 * 7900 / 1e9
    return res
