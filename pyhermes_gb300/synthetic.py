"""Seeded synthetic catalogues standing in for the reference's benchmark data
(the Quijote halo catalogue used by the reference docs is a download).

* ``uniform_catalogue``: uniform positions in a periodic box (float64).
* ``lognormal_catalogue``: a Gaussian field G with
  P(k) ~ k^-1.5 exp(-(k/k_s)^2) (k in h/Mpc, k_s = 0.5), normalised to
  sigma_G, density rho ~ exp(G - sigma_G^2/2), N points drawn with
  probability ~ rho per cell plus uniform in-cell jitter, clamped to
  [0, box); lognormal(0, sigma_w) weights.

Generation runs on the GPU with torch (it is set-up work, not the measured
path) and is deterministic for a given seed and device.
"""

import math

import numpy as np
import torch


def uniform_catalogue(n, box=1000.0, seed=0):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.0, box, (n, 3))


def gaussian_field(ng, box, sigma=1.0, k_smooth=0.5, slope=-1.5, seed=0, device="cuda"):
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    white = torch.randn((ng, ng, ng), generator=g, device=device, dtype=torch.float32)
    spec = torch.fft.rfftn(white)
    kf = 2.0 * math.pi / box
    kx = torch.fft.fftfreq(ng, d=1.0 / ng, device=device) * kf
    kz = torch.fft.rfftfreq(ng, d=1.0 / ng, device=device) * kf
    k2 = kx[:, None, None] ** 2 + kx[None, :, None] ** 2 + kz[None, None, :] ** 2
    k = torch.sqrt(k2)
    amp = torch.where(k > 0, k.clamp_min(1e-30) ** (slope / 2) * torch.exp(-0.5 * (k / k_smooth) ** 2),
                      torch.zeros_like(k))
    field = torch.fft.irfftn(spec * amp, s=(ng, ng, ng))
    field = field - field.mean()
    field = field * (sigma / field.std())
    return field


def lognormal_catalogue(n, box=1000.0, sigma_g=1.0, seed_field=0, seed_poisson=1, seed_weights=2,
                        sigma_w=0.3, ng=256, device="cuda"):
    """Returns (pos float64 (n,3) numpy, weights float64 (n,) numpy)."""
    G = gaussian_field(ng, box, sigma=sigma_g, seed=seed_field, device=device)
    rho = torch.exp(G.double() - 0.5 * sigma_g ** 2).reshape(-1)
    cdf = torch.cumsum(rho, 0)
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed_poisson))
    u = torch.rand(n, generator=gen, device=device, dtype=torch.float64) * cdf[-1]
    idx = torch.searchsorted(cdf, u).clamp_max(ng ** 3 - 1)
    ix = idx // (ng * ng)
    iy = (idx // ng) % ng
    iz = idx % ng
    jit = torch.rand((n, 3), generator=gen, device=device, dtype=torch.float64)
    cell = box / ng
    pos = torch.stack([ix, iy, iz], dim=1).double() * cell + jit * cell
    pos = pos.clamp(0.0, math.nextafter(box, 0.0))
    rng = np.random.default_rng(seed_weights)
    w = rng.lognormal(0.0, sigma_w, n)
    return pos.cpu().numpy(), w
