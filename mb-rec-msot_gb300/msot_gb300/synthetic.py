"""Seeded synthetic inputs (the reference loads measured data instead,
load_raw_data_for_reconstruction.m:8-15, which simulates with A as well).

  * gauss_pulse_eir: Gaussian-modulated cosine EIR (published gausspulse
    definition), centred, zero-padded to odd length.
  * phantom: disks (radius, amplitude uniform) plus Gaussian-profile line
    vessels, on a Discretization grid.
"""
from __future__ import annotations

import numpy as np


def gauss_pulse_eir(fs=4e7, fc=5e6, bw=0.6, n_taps=256, bwr_db=-6.0) -> np.ndarray:
    a = -(np.pi * fc * bw) ** 2 / (4.0 * np.log(10.0 ** (bwr_db / 20.0)))
    t = (np.arange(n_taps) - n_taps // 2) / fs
    e = np.exp(-a * t * t) * np.cos(2 * np.pi * fc * t)
    return np.concatenate([e, [0.0]]) if n_taps % 2 == 0 else e


def phantom(disc, rng: np.random.Generator, n_disks=(5, 15), r_disk=(0.3e-3, 3e-3),
            amp=(0.2, 1.0), n_vessels=3, vessel_width=0.2e-3) -> np.ndarray:
    """(nx, nz) image on the grid of ``disc`` (needs .x, .z, .fov)."""
    X, Z = np.meshgrid(disc.x, disc.z, indexing="ij")
    img = np.zeros(X.shape)
    x0, x1, z0, z1 = disc.fov
    half = 0.8 * min(x1 - x0, z1 - z0) / 2
    for _ in range(int(rng.integers(n_disks[0], n_disks[1] + 1))):
        cx, cz = rng.uniform(-half, half, 2)
        rad = rng.uniform(*r_disk)
        img[(X - cx) ** 2 + (Z - cz) ** 2 <= rad * rad] += rng.uniform(*amp)
    sig = vessel_width / 2.355
    for _ in range(n_vessels):
        px, pz = rng.uniform(-half, half, 2)
        th = rng.uniform(0, np.pi)
        across = -(X - px) * np.sin(th) + (Z - pz) * np.cos(th)
        along = (X - px) * np.cos(th) + (Z - pz) * np.sin(th)
        length = rng.uniform(0.3, 0.8) * (x1 - x0)
        img += (rng.uniform(*amp) * np.exp(-across ** 2 / (2 * sig * sig))
                * (np.abs(along) <= length / 2))
    return img


def phantom_batch(disc, count: int, seed: int = 0, device="cuda", n_disks=(5, 15),
                  r_disk=(0.3e-3, 3e-3), amp=(0.2, 1.0), n_vessels=3,
                  vessel_width=0.2e-3):
    """``count`` disk + vessel phantoms of ``phantom``'s distribution drawn on
    the device: (count, nx, nz) float32.  Unused disks get amplitude 0."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    u = lambda *s: torch.rand(*s, generator=g, device=device, dtype=torch.float64)
    X = torch.tensor(disc.x, device=device).view(1, -1, 1)
    Z = torch.tensor(disc.z, device=device).view(1, 1, -1)
    x0, x1, z0, z1 = disc.fov
    half = 0.8 * min(x1 - x0, z1 - z0) / 2
    img = torch.zeros((count, disc.nx, disc.nz), device=device, dtype=torch.float64)
    nd = n_disks[0] + (u(count) * (n_disks[1] - n_disks[0] + 1)).long()
    for k in range(n_disks[1]):
        cx, cz = (2 * u(count) - 1) * half, (2 * u(count) - 1) * half
        rad = r_disk[0] + u(count) * (r_disk[1] - r_disk[0])
        a = (amp[0] + u(count) * (amp[1] - amp[0])) * (k < nd)
        inside = ((X - cx.view(-1, 1, 1)) ** 2 + (Z - cz.view(-1, 1, 1)) ** 2
                  <= (rad ** 2).view(-1, 1, 1))
        img += a.view(-1, 1, 1) * inside
    sig = vessel_width / 2.355
    for _ in range(n_vessels):
        px, pz = [((2 * u(count) - 1) * half).view(-1, 1, 1) for _ in range(2)]
        th = (u(count) * np.pi).view(-1, 1, 1)
        across = -(X - px) * torch.sin(th) + (Z - pz) * torch.cos(th)
        along = (X - px) * torch.cos(th) + (Z - pz) * torch.sin(th)
        length = ((0.3 + 0.5 * u(count)) * (x1 - x0)).view(-1, 1, 1)
        a = (amp[0] + u(count) * (amp[1] - amp[0])).view(-1, 1, 1)
        img += a * torch.exp(-across ** 2 / (2 * sig * sig)) * (along.abs() <= length / 2)
    return img.to(torch.float32)
