"""Seeded synthetic models and acquisition geometries.

These stand in for the real-data workflow inputs (range.txt, station and
event catalogues, vel0 HDF5 files of scripts/sta_eve.jl and gene_vel0.jl),
which are not distributed with the reference.  All generators take a numpy
Generator and return FP64 arrays in the ops' C-order (m, n, l) layout, with
k the depth axis (k = 0 is the top surface).
"""
from __future__ import annotations

import numpy as np


def layered_checkerboard(m, n, l, block=8, amp=0.05, v_top=4.0, v_bot=8.0):
    """Velocity rising linearly from v_top to v_bot with depth, times a
    (1 +- amp) checkerboard of block-cell blocks.  Returns slowness (s/km)."""
    z = np.arange(l)
    v = v_top + (v_bot - v_top) * z / max(l - 1, 1)
    i = (np.arange(m) // block)[:, None, None]
    j = (np.arange(n) // block)[None, :, None]
    k = (np.arange(l) // block)[None, None, :]
    sgn = np.where((i + j + k) % 2 == 0, 1.0, -1.0)
    return 1.0 / (v[None, None, :] * (1.0 + amp * sgn))


def layered_smooth(m, n, l, rng, amp=0.05, v_top=4.0, v_bot=8.0, corr=6.0):
    """Layered velocity with a +-amp smooth random perturbation (Gaussian
    filtered white noise, correlation length `corr` cells).  Returns Vp."""
    z = np.arange(l)
    v = v_top + (v_bot - v_top) * z / max(l - 1, 1)
    noise = rng.standard_normal((m, n, l))
    # separable Gaussian smoothing via FFT
    spec = np.fft.rfftn(noise)
    kx = np.fft.fftfreq(m)[:, None, None]
    ky = np.fft.fftfreq(n)[None, :, None]
    kz = np.fft.rfftfreq(l)[None, None, :]
    spec *= np.exp(-2 * (np.pi * corr) ** 2 * (kx ** 2 + ky ** 2 + kz ** 2))
    sm = np.fft.irfftn(spec, s=(m, n, l), axes=(0, 1, 2))
    sm /= max(np.abs(sm).max(), 1e-30)
    return v[None, None, :] * (1.0 + amp * sm)


def gaussian_anomalies_2d(n1, m1, rng, v0=6.0, amp=0.1, sigma=8.0, count=3):
    """2D velocity: v0 background with `count` Gaussian anomalies of +-amp."""
    jj, ii = np.meshgrid(np.arange(n1), np.arange(m1), indexing="ij")
    v = np.full((n1, m1), v0)
    for _ in range(count):
        cj, ci = rng.uniform(sigma, n1 - sigma), rng.uniform(sigma, m1 - sigma)
        a = rng.choice([-amp, amp])
        v *= 1.0 + a * np.exp(-((jj - cj) ** 2 + (ii - ci) ** 2) / (2 * sigma ** 2))
    return v


def surface_stations(m, n, count, rng):
    """`count` receivers uniform on the top surface (k = 0)."""
    return np.column_stack([rng.uniform(0, m - 1, count), rng.uniform(0, n - 1, count),
                            np.zeros(count)])


def volume_sources(m, n, l, count, rng, margin=1.0):
    """`count` sources uniform in the volume (fractional node coordinates)."""
    return np.column_stack([rng.uniform(margin, m - 1 - margin, count),
                            rng.uniform(margin, n - 1 - margin, count),
                            rng.uniform(margin, l - 1 - margin, count)])
