"""Shared synthetic workloads for the tests (seeded; same shapes as the
benchmark configurations)."""
import numpy as np


def radial_c1_om():
    """2D radial: 256 spokes x 512 samples, angles k*pi/256, radius
    linspace(-pi, pi, 512, endpoint=False)."""
    ang = np.arange(256) * np.pi / 256
    rad = np.linspace(-np.pi, np.pi, 512, endpoint=False)
    om = np.empty((256 * 512, 2))
    om[:, 0] = (np.cos(ang)[:, None] * rad[None, :]).ravel()
    om[:, 1] = (np.sin(ang)[:, None] * rad[None, :]).ravel()
    return om


def cplx(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
