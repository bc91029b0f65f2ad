"""``density_to_stl`` of genpipeline/topology/mesh_export.py:7-67 with the surface extracted
on the device (gbsimp_marching_cubes) instead of skimage on the host.

Same threshold handling as the reference: ``None`` for an empty design (max < 0.01), the
level moved inside (min, max) by 10% of the range when it lies outside, and at least 0.1;
``ValueError`` when no surface is found. Vertices are in grid units times
``voxel_size_mm``. The file is a binary STL (80-byte header, triangle count, then per
triangle its unit normal, three vertices and a zero attribute word), the format numpy-stl
writes; normals follow the right-hand rule and point out of the solid.
"""
from __future__ import annotations

import numpy as np
import torch

_STL_DTYPE = np.dtype([("normal", "<f4", (3,)), ("v", "<f4", (3, 3)), ("attr", "<u2")])


def write_stl(path: str, tris: np.ndarray, header: bytes = b"genpipeline_gb300 density_to_stl") -> None:
    tris = np.asarray(tris, dtype=np.float32).reshape(-1, 3, 3)
    rec = np.zeros(len(tris), dtype=_STL_DTYPE)
    n = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0]).astype(np.float64)
    norm = np.linalg.norm(n, axis=1, keepdims=True)
    rec["normal"] = np.where(norm > 0, n / np.where(norm > 0, norm, 1.0), 0.0)
    rec["v"] = tris
    with open(path, "wb") as fh:
        fh.write(header[:80].ljust(80, b"\0"))
        fh.write(np.uint32(len(tris)).tobytes())
        fh.write(rec.tobytes())


def read_stl(path: str) -> np.ndarray:
    """(n, 3, 3) vertices of a binary STL written by write_stl."""
    with open(path, "rb") as fh:
        data = fh.read()
    n = int(np.frombuffer(data[80:84], dtype="<u4")[0])
    rec = np.frombuffer(data[84:84 + n * _STL_DTYPE.itemsize], dtype=_STL_DTYPE)
    return np.array(rec["v"])


def density_to_stl(density, output_path: str, threshold: float = 0.5,
                   voxel_size_mm: tuple = (100 / 32, 20 / 8, 20 / 8)):
    from ..engine import get_engine

    if isinstance(density, torch.Tensor):
        d = density.to(dtype=torch.float32).contiguous()
    else:
        if not torch.cuda.is_available():
            raise RuntimeError("density_to_stl extracts the surface on the GPU (no CPU fallback)")
        d = torch.as_tensor(np.ascontiguousarray(density, dtype=np.float32), device="cuda")
    dmin, dmax = float(d.min().item()), float(d.max().item())
    if dmax < 0.01:
        return None
    if threshold < dmin:
        threshold = dmin + 0.1 * (dmax - dmin)
    if threshold > dmax:
        threshold = dmax - 0.1 * (dmax - dmin)
    threshold = max(threshold, 0.1)
    tris = get_engine(d.device).marching_cubes(d, threshold, voxel_size_mm)
    if tris.shape[0] == 0:
        raise ValueError("density_to_stl: no surface found at threshold — check density field values")
    write_stl(output_path, tris.cpu().numpy())
    return output_path
