"""User window functions W(kx, ky, kz, *args) (k in cycles per cell) shared
by the golden generator and the custom-window tests.  They are plain Python:
the first two are elementwise NumPy code, the third only works on scalars
(``math`` calls and a branch), the fourth returns complex values."""
import math

import numpy as np


def aniso_gauss(kx, ky, kz, R, q=0.5):
    """Gaussian squashed along z by q."""
    return np.exp(-0.5 * (2.0 * np.pi * R) ** 2 * (kx * kx + ky * ky + (q * kz) ** 2))


def skewed_gauss(kx, ky, kz, R, shift=0.3):
    """Gaussian with a linear term in kx: not even in kx, so octant and
    full_rfft kernels differ."""
    return np.exp(-0.5 * (2.0 * np.pi * R) ** 2 * (kx * kx + ky * ky + kz * kz)) * (1.0 + shift * kx * R)


def stepped_tophat(kx, ky, kz, R):
    """Two-level step in |k| R, written for scalars only."""
    k = math.sqrt(kx * kx + ky * ky + kz * kz)
    if k * R < 0.15:
        return 1.0
    if k * R < 0.3:
        return 0.4
    return 0.05 * math.cos(k * R)


def odd_los(kx, ky, kz, R, nx, ny, nz):
    """i (n . k) 2 pi R times a Gaussian: an odd, complex directional window."""
    proj = (nx * kx + ny * ky + nz * kz) / math.sqrt(nx * nx + ny * ny + nz * nz)
    return 1j * 2.0 * np.pi * R * proj * np.exp(-0.5 * (2.0 * np.pi * R) ** 2 * (kx * kx + ky * ky + kz * kz))


def doubled_gauss(kx, ky, kz, R):
    """Twice a Gaussian: W(0) = 2, so a uniform random vertex behind it is a
    uniform field convolved with the window, not the bare density."""
    return 2.0 * np.exp(-0.5 * (2.0 * np.pi * R) ** 2 * (kx * kx + ky * ky + kz * kz))


def j0_shell(kx, ky, kz, R):
    """Thin spherical shell of radius R: j0(2 pi R |k|)."""
    return np.sinc(2.0 * R * np.sqrt(kx * kx + ky * ky + kz * kz))
