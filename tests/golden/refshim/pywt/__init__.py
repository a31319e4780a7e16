"""Stand-in for PyWavelets: ``Wavelet(name).wavefun(level)`` for orthogonal
wavelets, computed by the scaling-function cascade in ``pyhermes_gb300.phi``.
Parity with the real PyWavelets build is not pinned by this shim."""

import numpy as _np

from pyhermes_gb300.phi import scaling_cascade


class Wavelet:
    def __init__(self, name):
        self.name = name

    def wavefun(self, level=8):
        phi = scaling_cascade(self.name, level)
        x = _np.linspace(0.0, (phi.size - 1) / 2.0 ** level, phi.size)
        return phi, _np.zeros_like(phi), x
