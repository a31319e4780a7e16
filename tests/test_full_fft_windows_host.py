"""Complex full-FFT windows (io/window.py:198-264): legendre_multipole
(utils/legendre_windows.py) and radial_multipole
(utils/radial_multipole_windows.py:267-316) against the reference (golden
full_fft_windows_J4.npz): their kernels K_lm [L, L, L] and fields convolved
with them, ifftn(fftn(eps) K_lm).

On the host the oracle pins the golden kernels (1e-12) and stands in for
the multipole field kernels, so the window's parameter handling, the
impulse route to K and the `field @ W` dispatch run without a GPU
(complex64 output: 2e-6 of max|K|).  On the GPU the same cases run through
the CUDA field kernels: convolved fields within 2e-5 of max|value| (float32
FFTs), kernels within 1e-3 of max|K| (one more FFT of float32 data).
"""
import os

import numpy as np
import pytest
import torch
from scipy.fft import fftn, ifftn, irfftn

import oracle
from pyhermes_gb300 import multipole as mp
from pyhermes_gb300.phi import sample_scaling_function
from pyhermes_gb300.sfc_field import SFCField
from pyhermes_gb300.window import WindowFunc

PHI = sample_scaling_function()
SFC = {"J": 4, "box_size": 1000.0, "phi_resolution": 1024, "wavelet_mode": "db2", "wavelet_level": 10}
CASES = {
    "legendre_l2_m1": {"type": "legendre_multipole", "len_args": {"R": 150.0}, "other_args": {"l": 2, "m": 1}},
    "legendre_l3_mneg2": {"type": "legendre_multipole", "len_args": {"R": 120.0},
                          "other_args": {"l": 3, "m": -2, "use_fast": False}},
    "radial_thick_l2_mneg1": {"type": "radial_multipole", "len_args": {"R": 160.0, "delta_R": 60.0},
                              "other_args": {"radial_type": "thick_shell", "l": 2, "m": -1}},
    "radial_sphere_l0": {"type": "radial_multipole", "len_args": {"R": 140.0},
                         "other_args": {"radial_type": "sphere", "l": 0, "m": 0}},
    "radial_shell_l1_m1": {"type": "radial_multipole", "len_args": {"R": 180.0},
                           "other_args": {"radial_type": "shell", "l": 1, "m": 1}},
}
# oracle radial profile codes (shell 0, sphere 3) for the analytic cases
ORACLE_CODES = {"legendre_l2_m1": (0, "R"), "legendre_l3_mneg2": (0, "R"), "radial_sphere_l0": (3, "R"),
                "radial_shell_l1_m1": (0, "R")}


def _oracle_kernel(name, L=16):
    wp = CASES[name]
    code, key = ORACLE_CODES[name]
    P = oracle.fourier_power(PHI, 1, L)
    return oracle.radial_multipole_window(L, P, wp["len_args"][key] * L / 1000.0, wp["other_args"]["l"],
                                          wp["other_args"]["m"], code=code)


def _field(eps, device):
    f = SFCField(device=device)
    f.sfc_info = {**SFC, "L": 16, "V": 16 ** 3, "scale_factor": 16 / 1000.0, "field_kind": "derived_field",
                  "field_integral": float(eps.sum()), "phi_array": PHI, "phi_support": 3}
    f.format_sfc_params()
    f.epsilon = torch.as_tensor(eps, dtype=torch.float32, device=device)
    return f


def _rel(a, b):
    return np.abs(np.asarray(a) - b).max() / np.abs(b).max()


@pytest.mark.parametrize("name", sorted(ORACLE_CODES))
def test_oracle_matches_reference_full_fft_kernels(golden_dir, name):
    g = np.load(os.path.join(golden_dir, "full_fft_windows_J4.npz"))
    assert _rel(_oracle_kernel(name), g[name + "_kernel"]) < 1e-12


@pytest.fixture
def oracle_fields(monkeypatch):
    """multipole_fields_bins on the host: ifftn(fftn(eps) K) with the
    oracle's kernel for the single analytic bin of these windows."""
    def rfft_field(eps):
        return eps.detach().double().cpu().clone()

    def fields_bins(spec, J, l, m, bins, box, P, out=None, ws=None):
        L = 1 << J
        x = spec.numpy()
        eps = irfftn(x, s=(L,) * 3) if np.iscomplexobj(x) else x
        (b,) = bins
        code = {"shell": 0, "sphere": 3}[b.type]
        K = oracle.radial_multipole_window(L, oracle.fourier_power(PHI, 1, L), b.len_args["R"] * L / box, l, m,
                                           code=code)
        return torch.as_tensor(ifftn(fftn(eps) * K).ravel())

    monkeypatch.setattr(mp, "rfft_field", rfft_field)
    monkeypatch.setattr(mp, "multipole_fields_bins", fields_bins)


@pytest.mark.parametrize("name", sorted(ORACLE_CODES))
def test_full_fft_window_on_host(golden_dir, oracle_fields, name):
    g = np.load(os.path.join(golden_dir, "full_fft_windows_J4.npz"))
    w = WindowFunc(dict(CASES[name]), SFC, device="cpu")
    assert w.resolved_mode() == "complex_full_fft" and w.is_complex
    K = np.asarray(w.as_array())
    assert K.shape == (16, 16, 16) and _rel(K, g[name + "_kernel"]) < 2e-6
    conv = (_field(g["epsilon"], "cpu") @ w).epsilon
    assert np.iscomplexobj(conv) and _rel(conv, g[name + "_conv"]) < 2e-6


def test_full_fft_composite_on_host(golden_dir, oracle_fields):
    """A composite of two full-FFT windows keeps the [L, L, L] complex
    kernel and convolves with it (io/sfc_field.py:112-121)."""
    g = np.load(os.path.join(golden_dir, "full_fft_windows_J4.npz"))
    a = WindowFunc(dict(CASES["legendre_l2_m1"]), SFC, device="cpu")
    b = WindowFunc(dict(CASES["radial_shell_l1_m1"]), SFC, device="cpu")
    c = a - 0.5 * b
    ref_k = g["legendre_l2_m1_kernel"] - 0.5 * g["radial_shell_l1_m1_kernel"]
    assert _rel(c.as_array(), ref_k) < 2e-6
    conv = (_field(g["epsilon"], "cpu") @ c).epsilon
    ref = g["legendre_l2_m1_conv"] - 0.5 * g["radial_shell_l1_m1_conv"]
    assert _rel(conv, ref) < 2e-6


def test_full_fft_window_argument_rules():
    with pytest.raises(ValueError, match="bandwidth=1"):
        mp.complex_full_window_bin(WindowFunc(dict(CASES["legendre_l2_m1"]), SFC, bandwidth=2, device="cpu"))
    with pytest.raises(ValueError, match="missing required other_args"):
        mp.complex_full_window_bin(WindowFunc({"type": "legendre_multipole", "len_args": {"R": 100.0},
                                               "other_args": {"l": 2}}, SFC, device="cpu"))
    with pytest.raises(ValueError, match="requires len_args"):
        mp.complex_full_window_bin(WindowFunc({"type": "legendre_multipole", "other_args": {"l": 2, "m": 0}},
                                              SFC, device="cpu"))
    l, m, b = mp.complex_full_window_bin(WindowFunc(dict(CASES["radial_thick_l2_mneg1"]), SFC, device="cpu"))
    assert (l, m, b.type, b.len_args) == (2, -1, "thick_shell", {"R": 160.0, "delta_R": 60.0})
    with pytest.raises(ValueError, match="complex_full_fft"):
        WindowFunc(dict(CASES["legendre_l2_m1"], kernel_mode="octant"), SFC, device="cpu").resolved_mode()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_full_fft_window_gpu(golden_dir, name):
    g = np.load(os.path.join(golden_dir, "full_fft_windows_J4.npz"))
    w = WindowFunc(dict(CASES[name]), SFC)
    # K comes back through one forward FFT of the float32 impulse response,
    # which spreads its rounding over all L^3 modes: 1e-3 of max|K|
    assert _rel(np.asarray(w.as_array()), g[name + "_kernel"]) < 1e-3, name
    conv = (_field(g["epsilon"], "cuda") @ w).epsilon
    assert _rel(conv, g[name + "_conv"]) < 2e-5, name
