"""hermes_fft512_strided_inverse against a complex128 inverse FFT of the same
data (torch.fft.ifft times 512, unnormalised like CUFFT_INVERSE), on both
strided axes and both column tiles, and the J=9 multipole fields with the
own strided passes against cuFFT's 3-D plan.  Bound: 2e-6 of the largest
|value| of each field (FP32 rounding of a 512-point transform; cuFFT's own
FP32 result is held to the same bound)."""
import ctypes

import numpy as np
import pytest
import torch

from pyhermes_gb300 import _lib
from pyhermes_gb300 import multipole as mp
from pyhermes_gb300.kernels import _ptr, _stream_ptr
from pyhermes_gb300.phi import sample_scaling_function
from pyhermes_gb300.window import phi_power_device, rfft_field

pytestmark = pytest.mark.gpu
L = 512


@pytest.fixture(scope="module")
def data():
    g = torch.Generator(device="cuda").manual_seed(5)
    return torch.complex(torch.randn((2, L, L, L), device="cuda", generator=g),
                         torch.randn((2, L, L, L), device="cuda", generator=g))


@pytest.mark.parametrize("axis", [0, 1])
def test_strided_pass_matches_complex128_ifft(data, axis):
    x = data.clone()
    _lib.check(_lib.load().hermes_fft512_strided_inverse(_ptr(x), 2, axis, _stream_ptr(x.device)),
               "hermes_fft512_strided_inverse")
    for f in range(2):
        ref = torch.fft.ifft(data[f].to(torch.complex128), dim=axis) * L
        err = (x[f].to(torch.complex128) - ref).abs().max().item() / ref.abs().max().item()
        assert err <= 2e-6, (axis, f, err)
        del ref


def test_strided_pass_rejects_bad_arguments():
    lib = _lib.load()
    assert lib.hermes_fft512_strided_inverse(None, 1, 0, None) == -1
    buf = torch.empty(8, dtype=torch.complex64, device="cuda")
    for nf, axis in ((0, 0), (65, 0), (1, 2), (1, -1)):
        assert lib.hermes_fft512_strided_inverse(_ptr(buf), nf, axis, None) == -1


def test_fields_J9_own_strided_passes_match_cufft():
    lib = _lib.load()
    phi = sample_scaling_function()
    J = 9
    g = torch.Generator(device="cuda").manual_seed(1)
    spec = rfft_field(torch.randn((L, L, L), device="cuda", generator=g) * 1e-3)
    P = phi_power_device(phi, L, 1, 1024, "cuda")
    radii = [r * L / 1000.0 for r in np.linspace(10.0, 160.0, 6)]
    prev = lib.hermes_multipole_set_fft(0)
    try:
        ref = mp.multipole_fields(spec, J, 3, 2, radii, P, bin_major=True).clone()
        assert lib.hermes_multipole_set_fft(1) == 0
        got = mp.multipole_fields(spec, J, 3, 2, radii, P, bin_major=True)
        for b in range(len(radii)):
            err = (got[b] - ref[b]).abs().max().item() / ref[b].abs().max().item()
            assert err <= 2e-6, (b, err)
    finally:
        lib.hermes_multipole_set_fft(prev)
