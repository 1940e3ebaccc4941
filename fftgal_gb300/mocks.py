"""Lognormal mock catalogs with Zel'dovich velocities, generated on the GPU.

The clustered synthetic catalogs of the benchmark and training sets: a
Gaussian field g on an n^3 mesh with power spectrum
    P(k) = A (k / 0.1)^slope exp(-(k / 0.5)^2)   [Mpc/h]^3,
the lognormal density 1 + delta = exp(g - sigma^2 / 2), Poisson particle
counts per cell with uniform positions inside the cell, and the Zel'dovich
displacement Psi_k = i k / k^2 g_k sampled at each particle's cell.
Velocities are in the units gal_rsd takes with aH = 1 (src/gal.c:63-77):
v = f Psi, so the redshift-space catalog is x + (v . los) los.  Positions are
not wrapped (the paint wraps cells).  The same algorithm as
tests/golden/lognormal.py (numpy), with torch's generators.
"""
from __future__ import annotations

import math


def pk_model(k, amp: float = 1e4, slope: float = -1.5):
    import torch
    p = amp * torch.pow(torch.clamp(k, min=1e-30) / 0.1, slope) * torch.exp(-((k / 0.5) ** 2))
    return torch.where(k > 0, p, torch.zeros_like(p))


def lognormal_catalog(n: int, L: float, Np: float, seed: int, f: float = 0.8, slope: float = -1.5,
                      amp: float = 1e4, device=None, axes=(0, 1, 2)):
    """x, y, z, vx, vy, vz as FP32 tensors on ``device`` (default cuda) with
    about Np particles; velocity components not in ``axes`` are left None."""
    import torch
    dev = torch.device(device) if device is not None else torch.device("cuda")
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    kf = 2 * math.pi / L
    k1 = torch.fft.fftfreq(n, d=1.0 / n, device=dev, dtype=torch.float64) * kf
    kz = torch.fft.rfftfreq(n, d=1.0 / n, device=dev, dtype=torch.float64) * kf
    kx, ky, kzz = torch.meshgrid(k1, k1, kz, indexing="ij")
    k2 = kx * kx + ky * ky + kzz * kzz
    w = torch.randn((n, n, n), generator=gen, device=dev, dtype=torch.float32)
    # <|g_k|^2> = P(k) n^6 / L^3 for g_k = sum_x g(x) e^{-ikx}
    amp_k = torch.sqrt(pk_model(torch.sqrt(k2), amp, slope) * n ** 3 / L ** 3).to(torch.float32)
    gk = torch.fft.rfftn(w) * amp_k
    del w
    gk[0, 0, 0] = 0
    g = torch.fft.irfftn(gk, s=(n, n, n))
    sig2 = float(g.var())
    lam = (Np / n ** 3) * torch.clamp(torch.exp(g - 0.5 * sig2), min=0.0)
    del g
    counts = torch.poisson(lam.reshape(-1), generator=gen).to(torch.int64)
    del lam
    cell = torch.repeat_interleave(torch.arange(n ** 3, device=dev), counts)
    tot = int(cell.numel())
    H = L / n
    ci = cell // (n * n)
    cj = (cell // n) % n
    ck = cell % n
    x = ((ci.to(torch.float64) + torch.rand(tot, generator=gen, device=dev, dtype=torch.float64)) * H)
    y = ((cj.to(torch.float64) + torch.rand(tot, generator=gen, device=dev, dtype=torch.float64)) * H)
    z = ((ck.to(torch.float64) + torch.rand(tot, generator=gen, device=dev, dtype=torch.float64)) * H)
    inv = torch.where(k2 > 0, 1.0 / torch.clamp(k2, min=1e-300), torch.zeros_like(k2)).to(torch.float32)
    vel = []
    for a, kc in enumerate((kx, ky, kzz)):
        if a not in axes:
            vel.append(None)
            continue
        psi = torch.fft.irfftn(1j * kc.to(torch.float32) * inv * gk, s=(n, n, n))
        vel.append((f * psi.reshape(-1)[cell]).to(torch.float32))
        del psi
    return (x.to(torch.float32), y.to(torch.float32), z.to(torch.float32), vel[0], vel[1], vel[2])
