"""GPU window kernels, `field @ window` and Parseval 2PCF products against the
reference goldens and the float64 oracle.

Tolerances (float32 GPU vs float64 reference):
  * window kernels: |dK| <= 2e-6 * max|K|
  * convolved fields: |d| <= 1e-5 * max|ref|, relative L2 <= 2e-6
  * 2PCF products dd/dr/rr and xi: relative 1e-5 of max|product| over bins
"""
import os
import sys

import numpy as np
import pytest
import torch

import oracle
from pyhermes_gb300.phi import sample_scaling_function
from pyhermes_gb300.sfc_field import SFCField
from pyhermes_gb300.window import WindowFunc

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
from make_golden import WINDOW_CASES  # noqa: E402

pytestmark = pytest.mark.gpu
PHI = sample_scaling_function()


def _sfc(J):
    return {"J": J, "box_size": 1000.0, "phi_resolution": 1024, "wavelet_mode": "db2", "wavelet_level": 10}


@pytest.mark.parametrize("name", sorted(WINDOW_CASES))
def test_window_materialize_matches_reference(golden_dir, name):
    wp, bw = WINDOW_CASES[name]
    g = np.load(os.path.join(golden_dir, "windows_J4.npz"))[name]
    w = WindowFunc(dict(wp), _sfc(4), bandwidth=bw)
    k = w.as_array()
    assert k.shape == g.shape and np.iscomplexobj(k) == np.iscomplexobj(g)
    err = np.abs(k - g).max()
    assert err <= 2e-6 * np.abs(g).max(), (name, err, np.abs(g).max())


def _field_from(eps, J):
    f = SFCField()
    f.sfc_info = {**_sfc(J), "L": 1 << J, "V": (1 << J) ** 3, "scale_factor": (1 << J) / 1000.0,
                  "field_kind": "derived_field", "field_integral": float(eps.sum()), "phi_array": PHI,
                  "phi_support": 3}
    f.format_sfc_params()
    f.epsilon = torch.as_tensor(eps, dtype=torch.float32, device="cuda")
    return f


@pytest.mark.parametrize("name", ["gaussian", "thick_shell", "ring_tilted", "dirderiv", "inverse_laplacian"])
def test_convolution_matches_reference(golden_dir, name):
    d = np.load(os.path.join(golden_dir, "convolution_J5.npz"))
    f = _field_from(d["epsilon"], 5)
    w = WindowFunc(dict(WINDOW_CASES[name][0]), f.sfc_info)
    out = (f @ w).epsilon_device.double().cpu().numpy()
    ref = d["conv_" + name]
    assert np.abs(out - ref).max() <= 1e-5 * np.abs(ref).max()
    assert np.linalg.norm(out - ref) <= 2e-6 * np.linalg.norm(ref)


def test_composite_window_algebra():
    f = _field_from(np.random.default_rng(3).standard_normal((32, 32, 32)), 5)
    a = WindowFunc({"type": "gaussian", "len_args": {"R": 60.0}}, f.sfc_info)
    b = WindowFunc({"type": "shell", "len_args": {"R": 90.0}}, f.sfc_info)
    c = 2.0 * a - b
    out = (f @ c).epsilon_device
    ref = 2.0 * (f @ a).epsilon_device - (f @ b).epsilon_device
    assert torch.allclose(out, ref, atol=1e-5 * ref.abs().max().item())


def _corr_golden_field(d):
    from pyhermes_gb300.projection import SFCProjection

    return SFCProjection({"SFCProjection": {"particle_pos": d["pos"], "catalog_weight": d["weights"],
                                            "J": 5, "box_size": 1000.0}}).run(save_result=False)


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max()


def test_corr2pcf_matches_reference(golden_dir):
    from pyhermes_gb300.corr2pcf import Corr_2PCF

    d = np.load(os.path.join(golden_dir, "corr2pcf_J5.npz"))
    f = _corr_golden_field(d)
    task = Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform",
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": 40.0}, "mapping": "s_to_R"},
        "sampling": {"s": {"min": 60.0, "max": 300.0, "n": 5}},
        "products": ["dd", "dr", "delta_dd", "rr", "xi"]}})
    r = task.run(save_result=False)
    for k in ("dd", "dr", "rr", "delta_dd", "xi"):
        assert _rel(getattr(r, k), d["iso_" + k]) <= 1e-5, (k, _rel(getattr(r, k), d["iso_" + k]))
    task = Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform", "binning_window": {"type": "ring"},
        "sampling": {"s": {"min": 80.0, "max": 240.0, "n": 3}, "mu": {"min": 0.1, "max": 0.9, "n": 3}},
        "products": ["delta_dd", "xi"]}})
    r = task.run(save_result=False)
    assert r.xi.shape == (3, 3)
    assert _rel(r.delta_dd, d["smu_delta_dd"]) <= 1e-5
    assert _rel(r.xi, d["smu_xi"]) <= 1e-5
    task = Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform", "window": {"type": "gaussian", "len_args": {"R": 40.0}},
        "binning_window": {"type": "shell", "len_args": ["R"], "mapping": "s_to_R"},
        "sampling": {"s": {"min": 80.0, "max": 200.0, "n": 3}}, "products": ["xi"]}})
    r = task.run(save_result=False)
    assert _rel(r.xi, d["smooth_xi"]) <= 1e-5


def test_corr2pcf_cpu_config_200k_J7():
    """200,000 uniform points, J=7, 20 linear top-hat shells over 5-150 Mpc/h,
    random='uniform': xi against the float64 oracle (reference formulas)."""
    from pyhermes_gb300 import synthetic
    from pyhermes_gb300.corr2pcf import Corr_2PCF
    from pyhermes_gb300.projection import SFCProjection

    pos = synthetic.uniform_catalogue(200_000, seed=0)
    f = SFCProjection({"SFCProjection": {"particle_pos": pos, "J": 7, "box_size": 1000.0}}).run(save_result=False)
    edges = np.linspace(5.0, 150.0, 21)
    centers = 0.5 * (edges[1:] + edges[:-1])
    task = Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform",
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": float(edges[1] - edges[0])},
                           "mapping": "s_to_R"},
        "sampling": {"s": centers}, "products": ["dd", "delta_dd", "rr", "xi"]}})
    r = task.run(save_result=False)
    w = np.full(200_000, 1.0 / 200_000)
    eps = oracle.deposit(pos, w, PHI, 7, 1000.0)
    P = oracle.fourier_power(PHI, 1, 128)
    rho = 1.0 / 128 ** 3
    sf6 = (128 / 1000.0) ** 6
    ref_dd, ref_ddd = [], []
    for R in centers:
        K = oracle.window_kernel("thick_shell", {"R": R, "delta_R": 7.25}, 128, P)
        ref_dd.append(oracle.pair_product(eps, eps, K) * sf6)
        ref_ddd.append(oracle.pair_product(eps - rho, eps - rho, K) * sf6)
    ref_xi = np.array(ref_ddd) / (rho * rho * sf6)
    assert _rel(r.dd, ref_dd) <= 1e-5
    assert _rel(r.delta_dd, ref_ddd) <= 1e-5, _rel(r.delta_dd, ref_ddd)
    assert _rel(r.xi, ref_xi) <= 1e-5, _rel(r.xi, ref_xi)


def test_corr2pcf_random_field_matches_reference(golden_dir):
    """random = a projected random catalogue (dr, rd, rr and delta = D - R
    on the field paths): all products against the reference golden."""
    from pyhermes_gb300.corr2pcf import Corr_2PCF
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "random_catalogue_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                         "box_size": 1000.0}}).run(save_result=False)
    r = SFCProjection({"SFCProjection": {"particle_pos": g["rpos"], "J": 4, "box_size": 1000.0}}).run(
        save_result=False)
    d = Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": r,
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"},
        "sampling": {"s": {"min": 100.0, "max": 300.0, "n": 3}},
        "products": ["dd", "dr", "rd", "rr", "delta_dd", "xi"]}}).run(save_result=False)
    for k in ("dd", "dr", "rd", "rr", "delta_dd", "xi"):
        assert _rel(getattr(d, k), g["r2_" + k]) <= 1e-5, (k, getattr(d, k), g["r2_" + k])


@pytest.mark.parametrize("mode", ["raw", "field", "unit"])
def test_task_weight_normalization_matches_reference(golden_dir, mode):
    """Corr_2PCF products and Counting densities with the task-level
    weight_normalization on a catalogue field with field values."""
    from pyhermes_gb300.corr2pcf import Corr_2PCF
    from pyhermes_gb300.counting import Counting
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "normalization_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"],
                                         "field_value": g["field_value"], "J": 4, "box_size": 1000.0}}).run(
        save_result=False)
    d = Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform", "weight_normalization": mode,
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"},
        "sampling": {"s": {"min": 100.0, "max": 300.0, "n": 3}},
        "products": ["dd", "rr", "delta_dd", "xi"]}}).run(save_result=False)
    for k in ("dd", "rr", "delta_dd", "xi"):
        assert _rel(getattr(d, k), g[f"n2_{mode}_{k}"]) <= 1e-5, (mode, k)
    c = Counting({"Counting": {"sfc_field": f, "random_count": 400, "seed": 5,
                               "weight_normalization": mode}}).run(save_result=False)
    assert _rel(c.nx, g[f"count_{mode}_nx"]) <= 1e-5, mode


def test_corr2pcf_cross_fields_with_vertex_window_matches_reference(golden_dir):
    from pyhermes_gb300.corr2pcf import Corr_2PCF
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "cross_J4.npz"))
    a = SFCProjection({"SFCProjection": {"particle_pos": g["pa"], "catalog_weight": g["wa"], "J": 4,
                                         "box_size": 1000.0}}).run(save_result=False)
    b = SFCProjection({"SFCProjection": {"particle_pos": g["pb"], "J": 4, "box_size": 1000.0}}).run(
        save_result=False)
    d = Corr_2PCF({"Corr_2PCF": {
        "sfc_field1": a, "sfc_field2": b, "random": "uniform",
        "window1": {"type": "gaussian", "len_args": {"R": 30.0}},
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"},
        "sampling": {"s": {"min": 100.0, "max": 300.0, "n": 3}},
        "products": ["dd", "delta_dd", "xi"]}}).run(save_result=False)
    for k in ("dd", "delta_dd", "rr", "xi"):
        assert _rel(getattr(d, k), g["c2_" + k]) <= 1e-5, k


@pytest.mark.parametrize("kind", ["ring", "cylshell"])
def test_corr2pcf_rppi_sampling_matches_reference(golden_dir, kind):
    from pyhermes_gb300.corr2pcf import Corr_2PCF
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "rppi_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                         "box_size": 1000.0}}).run(save_result=False)
    d = Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform", "binning_window": {"type": kind, "mapping": "rppi_to_RH"},
        "sampling": {"rp": {"min": 60.0, "max": 180.0, "n": 3}, "pi": {"min": 30.0, "max": 90.0, "n": 2}},
        "products": ["delta_dd", "xi"]}}).run(save_result=False)
    for k in ("delta_dd", "xi"):
        assert _rel(getattr(d, k), g[f"{kind}_{k}"]) <= 1e-5, (kind, k)


def test_pair_product_at_sample_matches_reference(golden_dir):
    """compute_pair_product_at_sample / Corr_2PCF.calc_pair_product on the
    GPU (theory/corr2pcf.py:375-382, 632-645)."""
    from pyhermes_gb300 import corr2pcf
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "pair_at_sample_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "J": 4, "box_size": 1000.0}}).run(
        save_result=False)
    bw = {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"}
    v1 = corr2pcf.compute_pair_product_at_sample({"s": 150.0}, f, None, bw)
    task = corr2pcf.Corr_2PCF({"Corr_2PCF": {"sfc_field": f, "binning_window": bw, "sampling": {"s": [150.0]}}})
    v2 = task.calc_pair_product({"s": 220.0}, f)
    v3 = task.calc_pair_product({"s": 220.0}, f, 2.5e-4)
    np.testing.assert_allclose([v1, v2, v3], g["values"], rtol=1e-5)
