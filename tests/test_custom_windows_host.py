"""Window functions given as user callables (io/window.py:88-96, :274-332;
utils/convolution.py:14-283) against the reference (golden
custom_windows_J4.npz): the host-built kernel in full_rfft (the default),
octant, complex_rfft, auto and bandwidth 2, a function that only works on
scalars, a callable named with a built-in type; Corr_2PCF with a callable
binning window and a multipole task whose uniform random sits behind
windows with W(0) = 2 (on the host with the oracle's convolution, and on
the GPU); and, on the GPU, a field convolved with a custom window.

Tolerances: kernels are float64 on both sides, |dK| <= 1e-12 max|K|; the GPU
convolution is float32, |d| <= 1e-5 max|ref| and relative L2 <= 2e-6.
"""
import importlib.util
import os

import numpy as np
import pytest
import torch

import oracle
from pyhermes_gb300.window import WindowFunc, custom_window_kernel, ordered_window_args
from test_tasks_host import oracle_kernels  # noqa: F401  (fixture)

_spec = importlib.util.spec_from_file_location(
    "custom_window_funcs", os.path.join(os.path.dirname(__file__), "golden", "custom_window_funcs.py"))
cwf = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(cwf)

SFC = {"J": 4, "box_size": 1000.0, "phi_resolution": 1024, "wavelet_mode": "db2", "wavelet_level": 10}

CASES = {
    "gauss_full": ({"func": cwf.aniso_gauss, "len_args": {"R": 60.0}}, 1),
    "gauss_octant": ({"func": cwf.aniso_gauss, "len_args": {"R": 60.0}, "other_args": {"q": 0.7},
                      "kernel_mode": "octant"}, 1),
    "gauss_bw2": ({"func": cwf.aniso_gauss, "len_args": {"R": 40.0}}, 2),
    "skew_full": ({"func": cwf.skewed_gauss, "len_args": {"R": 50.0}}, 1),
    "skew_octant": ({"func": cwf.skewed_gauss, "len_args": {"R": 50.0}, "kernel_mode": "octant"}, 1),
    "skew_auto_axis": ({"func": cwf.skewed_gauss, "len_args": {"R": 50.0}, "kernel_mode": "auto",
                        "los_args": [0.0, 0.0, 1.0]}, 1),
    "step_full": ({"func": cwf.stepped_tophat, "len_args": {"R": 80.0}}, 1),
    "odd_complex": ({"func": cwf.odd_los, "len_args": {"R": 50.0}, "los_args": {"nx": 0.0, "ny": 1.0, "nz": 1.0},
                     "kernel_mode": "complex_rfft"}, 1),
    "named_gaussian": ({"type": "gaussian", "func": cwf.aniso_gauss, "len_args": {"R": 60.0}}, 1),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_custom_window_kernel_matches_reference(golden_dir, name):
    g = np.load(os.path.join(golden_dir, "custom_windows_J4.npz"))
    wp, bw = CASES[name]
    w = WindowFunc(dict(wp), SFC, bandwidth=bw, device="cpu")
    got = np.asarray(w.as_array())
    ref = g[name]
    assert [w.type, w.kernel_mode] == [str(v) for v in g[name + "_meta"]]
    assert got.shape == ref.shape and got.dtype == ref.dtype
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), name
    assert w.materialized and w.is_complex == np.iscomplexobj(ref)
    dev = w.kernel_device()
    assert dev.dtype == (torch.complex64 if np.iscomplexobj(ref) else torch.float32)


def test_custom_window_octant_and_full_agree_for_even_functions(golden_dir):
    g = np.load(os.path.join(golden_dir, "custom_windows_J4.npz"))
    # aniso_gauss is even on every axis: octant (with q = 0.7) differs from
    # full_rfft (q = 0.5) only through q; rebuild octant at q = 0.5 here
    w = WindowFunc({"func": cwf.aniso_gauss, "len_args": {"R": 60.0}, "kernel_mode": "octant"}, SFC, device="cpu")
    assert np.abs(w.as_array() - g["gauss_full"]).max() <= 1e-12
    # skewed_gauss is not: the reference's two modes differ and so do ours
    assert np.abs(g["skew_full"] - g["skew_octant"]).max() > 1e-3


def test_custom_window_argument_rules():
    def w3(kx, ky, kz, R, a, b=2.0):
        return R + a + b + 0.0 * kx
    assert ordered_window_args(w3, {"R": 1.0, "a": 3.0}) == [1.0, 3.0, 2.0]
    assert ordered_window_args(w3, {"R": 1.0, "a": 3.0, "b": 5.0, "extra": 9.0}) == [1.0, 3.0, 5.0]
    with pytest.raises(ValueError, match="Missing keyword arguments"):
        ordered_window_args(w3, {"R": 1.0})
    w = WindowFunc({"func": cwf.aniso_gauss}, SFC, device="cpu")
    with pytest.raises(ValueError, match="Missing keyword arguments"):
        w.as_array()
    with pytest.raises(TypeError):
        WindowFunc({"func": 3.0}, SFC, device="cpu")
    with pytest.raises(ValueError, match="complex_full_fft"):
        WindowFunc({"func": cwf.aniso_gauss, "len_args": {"R": 60.0}, "kernel_mode": "complex_full_fft"},
                   SFC, device="cpu").as_array()
    with pytest.raises(ValueError, match="descriptor"):
        WindowFunc({"func": cwf.aniso_gauss, "len_args": {"R": 60.0}}, SFC, device="cpu").descriptor()


def test_custom_window_scalar_fallback_equals_array_path():
    P = np.linspace(1.0, 0.2, 17)
    vec = custom_window_kernel(cwf.aniso_gauss, [1.5, 0.5], 16, 1, P, "full_rfft")
    scalar_only = custom_window_kernel(lambda kx, ky, kz, R, q: float(cwf.aniso_gauss(kx, ky, kz, R, q)),
                                       [1.5, 0.5], 16, 1, P, "full_rfft")
    assert np.abs(vec - scalar_only).max() <= 1e-15


def test_custom_window_composites(golden_dir):
    g = np.load(os.path.join(golden_dir, "custom_windows_J4.npz"))
    a = WindowFunc(dict(CASES["gauss_full"][0]), SFC, device="cpu")
    b = WindowFunc(dict(CASES["skew_full"][0]), SFC, device="cpu")
    c = a - 0.5 * b
    assert c.type == "composite" and not c.has_custom_func
    ref = g["gauss_full"] - 0.5 * g["skew_full"]
    assert np.abs(c.as_array() - ref).max() <= 1e-6 * np.abs(ref).max()


def test_window_copy(golden_dir):
    """WindowFunc.copy (io/window.py:487-516): the kernel copied or left to
    be rebuilt; composites refuse copy_kernel=False."""
    g = np.load(os.path.join(golden_dir, "custom_windows_J4.npz"))
    w = WindowFunc(dict(CASES["skew_full"][0]), SFC, device="cpu")
    k = w.as_array()
    c = w.copy()
    assert c.w_kernel is not k and np.array_equal(c.w_kernel, k) and c.func is w.func
    assert c._kernel_dev is not w._kernel_dev and torch.equal(c._kernel_dev, w._kernel_dev)
    c.w_kernel[0, 0, 0] = -1.0
    assert w.as_array()[0, 0, 0] != -1.0
    r = w.copy(copy_kernel=False)
    assert r.w_kernel is None and r._kernel_dev is None
    assert np.abs(r.as_array() - g["skew_full"]).max() <= 1e-12
    comp = w + r
    assert comp.copy().type == "composite"
    with pytest.raises(ValueError, match="copy_kernel=False"):
        comp.copy(copy_kernel=False)


@pytest.mark.gpu
def test_custom_window_convolution_matches_reference(golden_dir):
    from pyhermes_gb300.sfc_field import SFCField
    from pyhermes_gb300.phi import sample_scaling_function

    d = np.load(os.path.join(golden_dir, "custom_windows_J4.npz"))
    eps = d["epsilon"]
    f = SFCField()
    f.sfc_info = {**SFC, "L": 16, "V": 16 ** 3, "scale_factor": 16 / 1000.0, "field_kind": "derived_field",
                  "field_integral": float(eps.sum()), "phi_array": sample_scaling_function(), "phi_support": 3}
    f.format_sfc_params()
    f.epsilon = torch.as_tensor(eps, dtype=torch.float32, device="cuda")
    out = (f @ WindowFunc(dict(CASES["skew_full"][0]), f.sfc_info)).epsilon_device.double().cpu().numpy()
    ref = d["conv_skew"]
    assert np.abs(out - ref).max() <= 1e-5 * np.abs(ref).max()
    assert np.linalg.norm(out - ref) <= 2e-6 * np.linalg.norm(ref)


@pytest.mark.gpu
def test_uniform_random_behind_window_with_nonunit_zero_mode(golden_dir):
    """random = 'uniform' behind vertex windows with W(0) = 2: the random
    vertex is the uniform field convolved with the window
    (theory/corr3pcf_multipole.py:607-619), so rrr_l = (2 rho)^3 at l = 0."""
    g = np.load(os.path.join(golden_dir, "custom_windows_J4.npz"))
    d = _multipole_uniform_behind_w2(g, "cuda")
    for k in ("ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"):
        assert _rel(getattr(d, k), g["mp_" + k]) < 1e-4, k

@pytest.fixture
def numpy_convolution(monkeypatch):
    """field @ window on the host: the oracle's rFFT convolution with the
    window's own float64 kernel."""
    from pyhermes_gb300 import window as win_mod

    def apply_window(eps, w, out=None):
        K = np.asarray(w.as_array())
        return torch.as_tensor(oracle.convolve(eps.double().cpu().numpy(), K), dtype=torch.float32)

    monkeypatch.setattr(win_mod, "apply_window", apply_window)


def _rel(a, b):
    return np.abs(np.asarray(a) - b).max() / np.abs(b).max()


def _projected(g, device):
    from pyhermes_gb300.projection import SFCProjection

    return SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                            "box_size": 1000.0}}, device=device).run(save_result=False)


def _corr2pcf_custom_bins(g, device):
    from pyhermes_gb300.corr2pcf import Corr_2PCF

    return Corr_2PCF({"Corr_2PCF": {
        "sfc_field": _projected(g, device), "random": "uniform",
        "binning_window": {"func": cwf.j0_shell, "len_args": {"R": None}, "mapping": "s_to_R"},
        "sampling": {"s": {"min": 100.0, "max": 300.0, "n": 3}},
        "products": ["dd", "delta_dd", "xi"]}}, device=device).run(save_result=False)


def _multipole_uniform_behind_w2(g, device):
    from pyhermes_gb300.multipole import Corr_3PCF_Multipole

    win = {"type": "custom", "func": cwf.doubled_gauss, "len_args": {"R": 40.0}}
    return Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field": _projected(g, device), "random": "uniform",
        "window1": dict(win), "window2": dict(win), "window3": dict(win),
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [150.0, 200.0], "r13": [250.0, 300.0]},
        "l_min": 0, "l_max": 2, "products": ["ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"]}},
        device=device).run(save_result=False)


def test_corr2pcf_custom_binning_window_on_host(golden_dir, oracle_kernels, numpy_convolution):
    g = np.load(os.path.join(golden_dir, "custom_windows_J4.npz"))
    d = _corr2pcf_custom_bins(g, "cpu")
    for k in ("dd", "delta_dd", "rr", "xi"):
        assert _rel(getattr(d, k), g["c2_" + k]) < 1e-5, (k, getattr(d, k), g["c2_" + k])


def test_uniform_random_behind_nonunit_window_on_host(golden_dir, oracle_kernels, numpy_convolution):
    g = np.load(os.path.join(golden_dir, "custom_windows_J4.npz"))
    d = _multipole_uniform_behind_w2(g, "cpu")
    for k in ("ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"):
        assert _rel(getattr(d, k), g["mp_" + k]) < 1e-5, (k, getattr(d, k), g["mp_" + k])


@pytest.mark.gpu
def test_corr2pcf_custom_binning_window_gpu(golden_dir):
    g = np.load(os.path.join(golden_dir, "custom_windows_J4.npz"))
    d = _corr2pcf_custom_bins(g, "cuda")
    for k in ("dd", "delta_dd", "rr", "xi"):
        assert _rel(getattr(d, k), g["c2_" + k]) < 1e-4, k
