"""Seeded synthetic surfaces for the parity tests and the benchmark.

* noise_tilt: the LEM configurations' initial surface -- seeded uniform
  noise 0-1 m plus a planar tilt of `slope` toward the open edges,
  z += slope * dx * (cells to the nearest 'o'/'b' edge), the shape of the
  reference's generate_uniform_random_noise_surface +
  superimpose_open_boundary_gradient (synthetic_surfaces_cpu.cpp:359-459).
  The noise stream is numpy's, not the reference's hash; the oracle
  restates the reference's own stream where bit-equal inputs matter.
* fractal_pits: config 2 -- spectral synthesis with power spectrum ~ k^-2
  (random phases, amplitude k^-1), rescaled to the given relief, plus seeded
  paraboloid pits of uniform depth 0-5 m and radius 1-4 cells. The reference
  has no FFT on this machine (FFTW absent), so the surface is defined here.
"""
from __future__ import annotations

import numpy as np


def fractal(n_rows: int, n_cols: int, relief: float, seed: int, beta: float = 2.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    ky = np.fft.fftfreq(n_rows)[:, None]
    kx = np.fft.rfftfreq(n_cols)[None, :]
    k = np.sqrt(kx * kx + ky * ky)
    k[0, 0] = 1.0
    amp = k ** (-beta / 2.0)
    amp[0, 0] = 0.0
    phase = rng.uniform(0.0, 2.0 * np.pi, size=amp.shape)
    z = np.fft.irfft2(amp * np.exp(1j * phase), s=(n_rows, n_cols))
    z = (z - z.min()) / (z.max() - z.min()) * relief
    return z.astype(np.float32)


def add_pits(z: np.ndarray, n_pits: int, seed: int, rmin: float = 1.0, rmax: float = 4.0,
             dmax: float = 5.0) -> np.ndarray:
    rng = np.random.default_rng(seed + 1)
    nr, nc = z.shape
    cy = rng.integers(0, nr, n_pits)
    cx = rng.integers(0, nc, n_pits)
    rad = rng.uniform(rmin, rmax, n_pits)
    dep = rng.uniform(0.0, dmax, n_pits)
    z = z.copy()
    R = int(np.ceil(rmax))
    oy, ox = np.mgrid[-R:R + 1, -R:R + 1]
    dd = np.sqrt(oy * oy + ox * ox)
    for y, x, r, d in zip(cy, cx, rad, dep):
        w = np.clip(1.0 - (dd / r) ** 2, 0.0, None) * d
        y0, y1 = max(0, y - R), min(nr, y + R + 1)
        x0, x1 = max(0, x - R), min(nc, x + R + 1)
        z[y0:y1, x0:x1] -= w[y0 - (y - R):y1 - (y - R), x0 - (x - R):x1 - (x - R)].astype(np.float32)
    return z


def fractal_pits(n: int, relief: float = 1000.0, seed: int = 7, pits_per_8192sq: int = 100000) -> np.ndarray:
    z = fractal(n, n, relief, seed)
    return add_pits(z, max(1, int(round(pits_per_8192sq * (n / 8192.0) ** 2))), seed)


def noise_tilt(n_rows: int, n_cols: int, cell: float, seed: int, bc: str = "nnon", slope: float = 0.001) -> np.ndarray:
    rng = np.random.default_rng(seed)
    z = rng.random((n_rows, n_cols), dtype=np.float64)
    r = np.arange(n_rows)[:, None].astype(np.float64)
    c = np.arange(n_cols)[None, :].astype(np.float64)
    dist = np.full((n_rows, n_cols), np.inf)
    bc = (bc + "oooo")[:4].lower()
    if bc[0] in "ob":
        dist = np.minimum(dist, r + 0 * c)
    if bc[1] in "ob":
        dist = np.minimum(dist, (n_cols - 1 - c) + 0 * r)
    if bc[2] in "ob":
        dist = np.minimum(dist, (n_rows - 1 - r) + 0 * c)
    if bc[3] in "ob":
        dist = np.minimum(dist, c + 0 * r)
    if np.isfinite(dist).all():
        z = z + slope * cell * dist
    return z.astype(np.float32)


def fractal_subcritical(n_rows: int, n_cols: int, cell: float, critical_slope: float, seed: int,
                        target: float = 0.8, beta: float = 2.0):
    """A k^-2 fractal scaled so that its steepest slope -- the larger of the
    central-difference gradient magnitude and the face slope |dz|/dx over
    the whole grid -- is target * critical_slope: the Roering law is well
    posed on it everywhere (slopes at or above Sc have no feasible implicit
    step). Returns (z, relief in m)."""
    z = fractal(n_rows, n_cols, 1.0, seed, beta)
    smax = 0.0
    for r0 in range(0, n_rows, 2048):  # row bands keep the temporaries small
        w = z[max(0, r0 - 1):min(n_rows, r0 + 2049)].astype(np.float64)
        gx = (w[1:-1, 2:] - w[1:-1, :-2]) / (2.0 * cell)
        gy = (w[2:, 1:-1] - w[:-2, 1:-1]) / (2.0 * cell)
        smax = max(smax, float(np.sqrt(gx * gx + gy * gy).max()))
        smax = max(smax, float(np.abs(np.diff(w, axis=1)).max()) / cell, float(np.abs(np.diff(w, axis=0)).max()) / cell)
    scale = target * critical_slope / smax
    return (z * np.float32(scale)).astype(np.float32), scale
