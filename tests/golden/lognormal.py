"""Seeded lognormal mock catalogs with Zel'dovich velocities (test input).

The clustered catalog of the folded-box configuration: a Gaussian field with
P(k) = 1e4 (k/0.1)^-1.5 exp(-(k/0.5)^2) [Mpc/h]^3 on an n^3 mesh, the lognormal
transform 1 + delta = exp(g - sigma^2/2), Poisson particle counts per cell with
uniform positions inside the cell, and Zel'dovich displacements
Psi_k = i k / k^2 g_k.  Velocities are returned in the units gal_rsd expects
with aH = 1 (src/gal.c:63-77): v = f Psi, so a redshift-space catalog is
x + (v . los) los.  Positions are not wrapped (the paint wraps cells).
"""
from __future__ import annotations

import numpy as np


def pk_model(k: np.ndarray) -> np.ndarray:
    with np.errstate(divide="ignore"):
        p = 1e4 * (k / 0.1) ** -1.5 * np.exp(-((k / 0.5) ** 2))
    p[k == 0] = 0.0
    return p


def lognormal_catalog(seed: int, n: int, L: float, Np: float, f: float = 0.8):
    """Return x, y, z, vx, vy, vz (float64) of about Np particles."""
    rng = np.random.default_rng(seed)
    kf = 2 * np.pi / L
    k1 = np.fft.fftfreq(n, d=1.0 / n) * kf
    kz = np.fft.rfftfreq(n, d=1.0 / n) * kf
    kx, ky, kzz = np.meshgrid(k1, k1, kz, indexing="ij")
    k2 = kx ** 2 + ky ** 2 + kzz ** 2
    kk = np.sqrt(k2)
    # white noise -> field with <|g_k|^2> = P(k) n^6 / L^3 (g_k = sum_x g(x) e^{-ikx})
    w = rng.standard_normal((n, n, n))
    gk = np.fft.rfftn(w) * np.sqrt(pk_model(kk) * n ** 3 / L ** 3)
    gk[0, 0, 0] = 0.0
    g = np.fft.irfftn(gk, s=(n, n, n), axes=(0, 1, 2))
    sig2 = g.var()
    dln = np.exp(g - 0.5 * sig2) - 1.0
    nbar_cell = Np / n ** 3
    counts = rng.poisson(nbar_cell * np.clip(1.0 + dln, 0.0, None))
    tot = int(counts.sum())
    cell = np.repeat(np.arange(n ** 3), counts.ravel())
    ci, cj, ck = np.unravel_index(cell, (n, n, n))
    H = L / n
    x = (ci + rng.random(tot)) * H
    y = (cj + rng.random(tot)) * H
    z = (ck + rng.random(tot)) * H
    # Zel'dovich displacement field, sampled at each particle's cell
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = np.where(k2 > 0, 1.0 / k2, 0.0)
    vel = []
    for kc in (kx, ky, kzz):
        psi = np.fft.irfftn(1j * kc * inv * gk, s=(n, n, n), axes=(0, 1, 2))
        vel.append(f * psi.ravel()[cell])
    return x, y, z, vel[0], vel[1], vel[2]
