"""Seeded synthetic trajectories and images for the benchmark workloads.

The reference ships one 2D trajectory (src/data/om2D.npz) and a phantom; these
generators produce the shapes the benchmark configurations name, in
normalised radians (om in [-pi, pi)), as float64 (M, ndim) arrays.
"""
from __future__ import annotations

import numpy as np


def radial_2d(spokes: int = 256, samples: int = 512, golden: bool = False) -> np.ndarray:
    """Radial spokes through the centre: angle k*pi/spokes (or the golden-angle
    increment pi*(sqrt(5)-1)/2), radius linspace(-pi, pi, samples, endpoint=False)."""
    k = np.arange(spokes)
    ang = (k * np.pi * (np.sqrt(5) - 1) / 2) % np.pi if golden else k * np.pi / spokes
    rad = np.linspace(-np.pi, np.pi, samples, endpoint=False)
    om = np.empty((spokes * samples, 2))
    om[:, 0] = (np.cos(ang)[:, None] * rad[None, :]).ravel()
    om[:, 1] = (np.sin(ang)[:, None] * rad[None, :]).ravel()
    return om


def uniform(M: int, ndim: int, seed: int) -> np.ndarray:
    """i.i.d. uniform points in [-pi, pi)^ndim."""
    return np.random.default_rng(seed).uniform(-np.pi, np.pi, (M, ndim))


def spiral_2d(interleaves: int = 32, samples: int = 2048, power: float = 1.5,
              turns: float = 16.0, seed: int = 6) -> np.ndarray:
    """Variable-density spiral: r = pi * t^power, theta = 2 pi turns t + the
    interleaf rotation, t in [0, 1); a seeded global rotation."""
    rng = np.random.default_rng(seed)
    rot0 = rng.uniform(0, 2 * np.pi)
    t = np.arange(samples) / samples
    r = np.pi * t ** power
    th = 2 * np.pi * turns * t
    om = np.empty((interleaves * samples, 2))
    for i in range(interleaves):
        a = th + rot0 + 2 * np.pi * i / interleaves
        om[i * samples:(i + 1) * samples, 0] = r * np.cos(a)
        om[i * samples:(i + 1) * samples, 1] = r * np.sin(a)
    return np.clip(om, -np.pi, np.pi - 1e-12)


def kooshball_3d(spokes: int = 15625, samples: int = 512) -> np.ndarray:
    """3D radial: spoke directions on a Fibonacci sphere, samples along each
    spoke at radius linspace(-pi, pi, samples, endpoint=False)."""
    i = np.arange(spokes) + 0.5
    phi = np.arccos(1 - 2 * i / spokes)
    theta = np.pi * (1 + 5 ** 0.5) * i
    d = np.stack([np.cos(theta) * np.sin(phi), np.sin(theta) * np.sin(phi), np.cos(phi)], 1)
    rad = np.linspace(-np.pi, np.pi, samples, endpoint=False)
    return (d[:, None, :] * rad[None, :, None]).reshape(-1, 3)


def random_image(shape, seed: int = 0) -> np.ndarray:
    """complex64 image with real and imaginary parts i.i.d. N(0, 1)."""
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def ellipsoids(shape, count: int = 32, seed: int = 2) -> np.ndarray:
    """Sum of `count` ellipsoids: uniform centres inside the field of view,
    semi-axes uniform in [0.05, 0.3] * N, complex N(0, 1) amplitudes."""
    rng = np.random.default_rng(seed)
    shape = tuple(shape)
    grids = np.meshgrid(*[np.arange(n, dtype=np.float32) for n in shape], indexing='ij')
    img = np.zeros(shape, dtype=np.complex64)
    for _ in range(count):
        c = [rng.uniform(0.2 * n, 0.8 * n) for n in shape]
        ax = [rng.uniform(0.05 * n, 0.3 * n) for n in shape]
        amp = np.complex64(rng.standard_normal() + 1j * rng.standard_normal())
        q = sum(((g - ci) / ai) ** 2 for g, ci, ai in zip(grids, c, ax))
        img[q <= 1.0] += amp
    return img


def add_noise(y: np.ndarray, snr_db: float, seed: int) -> np.ndarray:
    """y + complex Gaussian noise at the given SNR (power ratio in dB)."""
    rng = np.random.default_rng(seed)
    p = np.mean(np.abs(y) ** 2)
    sigma = np.sqrt(p / 10 ** (snr_db / 10) / 2)
    n = sigma * (rng.standard_normal(y.shape) + 1j * rng.standard_normal(y.shape))
    return (y + n).astype(np.complex64)


def coil_maps(shape2d, coils: int = 32, seed: int = 4) -> np.ndarray:
    """Smooth complex Gaussian sensitivities (sigma 0.3 N) centred on a ring of
    radius 0.35 N, random phases: (Nx, Ny, coils) complex64."""
    rng = np.random.default_rng(seed)
    nx, ny = shape2d
    X, Y = np.meshgrid(np.arange(nx) - nx / 2, np.arange(ny) - ny / 2, indexing='ij')
    out = np.empty((nx, ny, coils), dtype=np.complex64)
    for c in range(coils):
        a = 2 * np.pi * c / coils
        cx, cy = 0.35 * nx * np.cos(a), 0.35 * ny * np.sin(a)
        g = np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * (0.3 * nx) ** 2))
        out[..., c] = g * np.exp(1j * rng.uniform(0, 2 * np.pi))
    return out


def uneven_instances(count: int = 64, lo: int = 20000, hi: int = 200000, seed: int = 5):
    """`count` independent 2D uniform trajectories with M ~ U{lo..hi}."""
    rng = np.random.default_rng(seed)
    Ms = rng.integers(lo, hi + 1, size=count)
    return [rng.uniform(-np.pi, np.pi, (int(m), 2)) for m in Ms]
