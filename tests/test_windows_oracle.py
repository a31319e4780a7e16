"""Oracle window kernels, convolution and pair products against the
reference's outputs (golden fixtures), float64 to rounding."""
import os
import sys

import numpy as np
import pytest

import oracle

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
from make_golden import WINDOW_CASES  # noqa: E402


def _mode(name, wp):
    if wp["type"] == "directional_derivative":
        return "complex_rfft"
    if name == "ring_tilted":
        return "full_rfft"
    return "octant"


def _los(wp):
    los = wp.get("los_args", {})
    return (los["nx"], los["ny"], los["nz"]) if los else (0.0, 0.0, 1.0)


@pytest.fixture(scope="module")
def phi(golden_dir):
    return np.load(os.path.join(golden_dir, "phi_db2.npz"))["phi"]


@pytest.mark.parametrize("name", sorted(WINDOW_CASES))
def test_oracle_window_kernel_matches_reference(golden_dir, phi, name):
    wp, bw = WINDOW_CASES[name]
    g = np.load(os.path.join(golden_dir, "windows_J4.npz"))[name]
    P = oracle.fourier_power(phi, bw, 16 * bw)
    k = oracle.window_kernel(wp["type"], wp.get("len_args", {}), 16, P, mode=_mode(name, wp), los=_los(wp),
                             bandwidth=bw)
    assert k.dtype == g.dtype
    np.testing.assert_allclose(k, g, rtol=0, atol=1e-14 * max(1.0, np.abs(g).max()))


def test_oracle_convolution_and_pair_product(golden_dir, phi):
    d = np.load(os.path.join(golden_dir, "convolution_J5.npz"))
    P = oracle.fourier_power(phi, 1, 32)
    for name in ("gaussian", "thick_shell", "ring_tilted", "dirderiv", "inverse_laplacian"):
        wp = WINDOW_CASES[name][0]
        K = oracle.window_kernel(wp["type"], wp.get("len_args", {}), 32, P, mode=_mode(name, wp), los=_los(wp))
        conv = oracle.convolve(d["epsilon"], K)
        ref = d["conv_" + name]
        np.testing.assert_allclose(conv, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
