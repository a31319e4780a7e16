"""The scaling function's precomputes on the device (hermes_phi_prepare)
against the host restatements pinned to the reference (phi.fourier_power_spectrum,
phi.cal_gamma): float64, 1e-12 relative."""
import ctypes

import numpy as np
import pytest
import torch

from pyhermes_gb300 import _lib
from pyhermes_gb300.kernels import _ptr, _stream_ptr
from pyhermes_gb300.phi import cal_gamma, fourier_power_spectrum, sample_scaling_function

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("L,bw", [(32, 1), (512, 1), (64, 2)])
def test_phi_prepare_matches_host(L, bw):
    phi = sample_scaling_function()
    pt = torch.as_tensor(phi, device="cuda")
    power = torch.empty(L * bw + 1, dtype=torch.float64, device="cuda")
    gamma = torch.empty(9, dtype=torch.float64, device="cuda")
    _lib.check(_lib.load().hermes_phi_prepare(_ptr(pt), phi.size, 1024, L, bw, _ptr(power), _ptr(gamma),
                                              _stream_ptr()), "hermes_phi_prepare")
    want = fourier_power_spectrum(phi, bw, L * bw, 1024)
    np.testing.assert_allclose(power.cpu().numpy(), want, rtol=1e-12, atol=1e-14 * want.max())
    np.testing.assert_allclose(gamma.cpu().numpy().reshape(3, 3), cal_gamma(phi, 3, 1024), rtol=1e-12, atol=1e-15)
