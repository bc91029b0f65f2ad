"""Seeded synthetic densities and load cases of the batched and serving workloads (host).

Density field: white noise N(0, 1) from numpy's PCG64(seed), FFT-convolved with a Gaussian
of standard deviation 6 voxels (periodic), normalised to zero mean and unit standard
deviation, passed through a sigmoid, scaled so that its mean equals m ~ U(0.2, 0.5) (drawn
from the same generator after the noise) and clipped to [1e-3, 1].
"""
from __future__ import annotations

import numpy as np

from . import bcs


def grf_density(grid, seed: int, length_scale: float = 6.0) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    nx, ny, nz = grid
    w = rng.standard_normal((nx, ny, nz))
    m = rng.uniform(0.2, 0.5)
    k = [np.fft.fftfreq(n) for n in (nx, ny, nz)]
    kx, ky, kz = np.meshgrid(*k, indexing="ij")
    # Fourier transform of a unit-mass Gaussian of std s (voxels): exp(-2 pi^2 s^2 |k|^2)
    g = np.exp(-2.0 * np.pi ** 2 * length_scale ** 2 * (kx ** 2 + ky ** 2 + kz ** 2))
    z = np.real(np.fft.ifftn(np.fft.fftn(w) * g))
    z = (z - z.mean()) / (z.std() + 1e-30)
    s = 1.0 / (1.0 + np.exp(-z))
    x = s * (m / s.mean())
    return np.clip(x, 1e-3, 1.0).astype(np.float32)


def cantilever_case(n: int):
    """Cantilever scaled to an n^3 grid: x = 0 clamped, unit -z point load at (n, n/2, 0)."""
    return bcs.cantilever_tip(n, n, n)


LOADS = ("cantilever", "top_patch", "torsion")


def load_case(name: str, n: int):
    if name == "cantilever":
        return bcs.cantilever_tip(n, n, n)
    if name == "top_patch":
        return bcs.top_patch(n, n, n)
    if name == "torsion":
        return bcs.torsion_couple(n, n, n)
    raise ValueError(name)


def _grf_field(shape, seed: int, length_scale: float) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    w = rng.standard_normal(shape)
    k = [np.fft.fftfreq(n) for n in shape]
    kx, ky, kz = np.meshgrid(*k, indexing="ij")
    g = np.exp(-2.0 * np.pi ** 2 * length_scale ** 2 * (kx ** 2 + ky ** 2 + kz ** 2))
    z = np.real(np.fft.ifftn(np.fft.fftn(w) * g))
    return (z - z.mean()) / (z.std() + 1e-30)


class LatentFieldDecoder:
    """A stand-in for the VAE decoder that the evaluator calls (the VAE itself is not part of
    this package): ``decode(z)`` maps latent vectors (B, latent_dim) to densities
    (B, 1, size, size, size) = sigmoid(gain * sum_k z_k F_k), where F_k are fixed seeded
    Gaussian random fields (``_grf_field`` with PCG64(seed + k)). Deterministic, on the
    device, with the ``parameters()`` / ``decode`` interface the evaluator uses."""

    def __init__(self, latent_dim: int = 16, size: int = 64, seed: int = 0, length_scale: float = 6.0,
                 gain: float = 1.5, device="cuda"):
        import torch

        f = np.stack([_grf_field((size, size, size), seed + k, length_scale) for k in range(latent_dim)])
        self.fields = torch.as_tensor(f.reshape(latent_dim, -1), dtype=torch.float32, device=device)
        self.latent_dim, self.size, self.gain = latent_dim, size, gain

    def parameters(self):
        return iter([self.fields])

    def decode(self, z):
        import torch

        z = torch.as_tensor(z, dtype=torch.float32, device=self.fields.device).reshape(-1, self.latent_dim)
        v = torch.sigmoid(self.gain * (z @ self.fields) / np.sqrt(self.latent_dim))
        return v.reshape(-1, 1, self.size, self.size, self.size)
