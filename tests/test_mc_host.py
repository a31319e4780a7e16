"""Host-side assembly of the Monte Carlo 3PCF products (no GPU):
``Corr_3PCF`` with its triplet kernel replaced by a float64 CPU sum of the
oracle's 27-point interpolation, against the reference's particle-centre
golden (explicit random centres): ddd, rrr, d_delta_dd, r_delta_dd and
delta_ddd = d_delta_dd - r_delta_dd, relative 1e-5 (the field is read as
float32, as on the GPU)."""
import os

import numpy as np
import pytest
import torch

import oracle
from pyhermes_gb300 import mc3pcf
from pyhermes_gb300.phi import sample_scaling_function
from pyhermes_gb300.sfc_field import SFCField
from test_tasks_host import oracle_kernels  # noqa: F401  (fixture: oracle pair products for xi23)

PHI = sample_scaling_function()


def _cpu_triplet_sum(eps1, eps2, eps3, J, centers, offsets, phi_t, center_w=None, rho1=0.0, samples=False,
                     locality=True):
    c = centers.double().cpu().numpy() if isinstance(centers, torch.Tensor) else np.asarray(centers, np.float64)
    phi = phi_t.double().cpu().numpy()
    e2, e3 = (e.double().cpu().numpy() for e in (eps2, eps3))
    n1 = oracle.interp(c, eps1.double().cpu().numpy(), phi, J) if eps1 is not None else rho1
    w = np.ones(c.shape[0]) if center_w is None else np.asarray(center_w, dtype=np.float64)
    total = 0.0
    for o in np.asarray(offsets, dtype=np.float64):
        n2 = oracle.interp(c, e2, phi, J, offset=o[0:3])
        n3 = oracle.interp(c, e3, phi, J, offset=o[3:6])
        total += float(np.sum(w * n1 * n2 * n3))
    return total, None


def _golden_field(g):
    J, L = 4, 16
    f = SFCField(device="cpu")
    f.sfc_info = {"J": J, "L": L, "V": L ** 3, "box_size": 1000.0, "scale_factor": L / 1000.0,
                  "phi_resolution": 1024, "wavelet_mode": "db2", "wavelet_level": 10, "phi_array": PHI,
                  "phi_support": 3, "field_kind": "derived_field", "field_integral": float(g["field_integral"])}
    f.format_sfc_params()
    f.epsilon = torch.as_tensor(g["epsilon"], dtype=torch.float32)
    return f


def _rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / np.abs(b).max()


def test_particle_centre_products_match_reference(golden_dir, oracle_kernels, monkeypatch):
    g = np.load(os.path.join(golden_dir, "mc3pcf_particle_J4.npz"))
    monkeypatch.setattr(mc3pcf, "triplet_sum", _cpu_triplet_sum)
    task = mc3pcf.Corr_3PCF({"Corr_3PCF": {
        "sfc_field": _golden_field(g), "random": "uniform", "r12": 150.0, "r13": 250.0, "angle_param": "mu",
        "mu": {"mu_min": -0.8, "mu_max": 0.8, "n_mu": 3}, "n_rot": 3, "center": "particle", "base_seed": 7,
        "particle_pos1": g["cpos"], "particle_weight1": g["cw"], "random_pos1": g["rpos"], "random_weight1": g["rw"],
        "products": ["ddd", "rrr", "d_delta_dd", "r_delta_dd", "delta_ddd"]}}, device="cpu")
    d = task.run()
    np.testing.assert_allclose(d.mu, g["rpos_mu"])
    for k in ("ddd", "rrr", "d_delta_dd", "r_delta_dd", "delta_ddd"):
        assert _rel(getattr(d, k), g["rpos_" + k]) < 1e-5, (k, getattr(d, k), g["rpos_" + k])


def test_particle_centre_argument_rules():
    base = {"sfc_field": "", "r12": 150.0, "r13": 250.0, "center": "particle", "products": ["ddd"]}
    t = mc3pcf.Corr_3PCF({"Corr_3PCF": dict(base, products=["zeta"])}, device="cpu")
    assert {"delta_ddd", "d_delta_dd", "r_delta_dd", "rrr"} <= set(t.expanded)
    with pytest.raises(ValueError):  # box-random centres have no d_delta_dd
        mc3pcf.Corr_3PCF({"Corr_3PCF": dict(base, center="box_random", products=["d_delta_dd"])}, device="cpu")
    with pytest.raises(ValueError):  # positions and weights come together
        mc3pcf._centre_arrays(np.zeros((3, 3)), None, "particle_pos1", "particle_weight1")
    with pytest.raises(ValueError):
        mc3pcf._centre_arrays(np.zeros((3, 3)), np.zeros(3), "particle_pos1", "particle_weight1")
    with pytest.raises(ValueError):
        mc3pcf._centre_arrays(np.zeros((3, 2)), np.ones(3), "particle_pos1", "particle_weight1")


def test_box_random_products_match_reference(golden_dir, oracle_kernels, monkeypatch):
    """center='box_random' (seeded box centres, n1 interpolated): ddd, rrr
    and delta_ddd against the reference golden, with the field deposited by
    the oracle from the same catalogue (catalog weight normalisation)."""
    g = np.load(os.path.join(golden_dir, "mc3pcf_J4.npz"))
    pw, integral = oracle.projection_weights(g["weights"], np.ones_like(g["weights"]), "catalog")
    eps = oracle.deposit(g["pos"], pw, PHI, 4, 1000.0)
    monkeypatch.setattr(mc3pcf, "triplet_sum", _cpu_triplet_sum)
    d = mc3pcf.Corr_3PCF({"Corr_3PCF": {
        "sfc_field": _golden_field({"epsilon": eps, "field_integral": integral}), "random": "uniform",
        "r12": 150.0, "r13": 250.0, "angle_param": "mu", "mu": {"mu_min": -0.8, "mu_max": 0.8, "n_mu": 3},
        "n_rot": 3, "center": "box_random", "n_box_centers": 600, "base_seed": 42,
        "products": ["ddd", "rrr", "delta_ddd"]}}, device="cpu").run()
    for k in ("ddd", "rrr", "delta_ddd"):
        assert _rel(getattr(d, k), g["box_" + k]) < 1e-5, (k, getattr(d, k), g["box_" + k])


def test_particle_centre_products_with_windows(golden_dir, oracle_kernels, monkeypatch):
    """Smoothing windows on the MC vertices (a shared gaussian and a sphere
    on vertex 3): the windowed data fields, the uniform random as the
    windowed field's mean density, xi23 and zeta (theory/corr3pcf.py:176-183,
    1038-1104); convolutions by the oracle on the host."""
    from pyhermes_gb300 import window as win_mod
    from pyhermes_gb300.projection import SFCProjection

    def apply_window(eps, w, out=None):
        K = oracle.window_kernel(w.type, w.len_args, w.L, oracle.fourier_power(PHI, w.bandwidth, w.L),
                                 mode=w.resolved_mode(), box=w.box_size)
        return torch.as_tensor(oracle.convolve(eps.double().cpu().numpy(), K), dtype=torch.float32)

    monkeypatch.setattr(win_mod, "apply_window", apply_window)
    monkeypatch.setattr(mc3pcf, "triplet_sum", _cpu_triplet_sum)
    g = np.load(os.path.join(golden_dir, "mc3pcf_particle_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                         "box_size": 1000.0}}, device="cpu").run(save_result=False)
    d = mc3pcf.Corr_3PCF({"Corr_3PCF": {
        "sfc_field": f, "random": "uniform", "r12": 150.0, "r13": 250.0, "angle_param": "mu",
        "mu": {"mu_min": -0.8, "mu_max": 0.8, "n_mu": 3}, "n_rot": 3, "center": "particle", "base_seed": 7,
        "particle_pos1": g["cpos"], "particle_weight1": g["cw"],
        "window": {"type": "gaussian", "len_args": {"R": 40.0}},
        "window3": {"type": "sphere", "len_args": {"R": 60.0}},
        "products": ["zeta", "ddd"]}}, device="cpu").run(save_result=False)
    for k in ("ddd", "rrr", "d_delta_dd", "r_delta_dd", "delta_ddd", "xi23", "zeta"):
        assert _rel(getattr(d, k), g["win_" + k]) < 1e-5, (k, getattr(d, k), g["win_" + k])
    info = d.corr3pcf_info
    # merged over the defaults; each window keeps its own len_args
    assert info["window1"] == info["window2"] == {"type": "gaussian", "len_args": {"R": 40.0}, "los_args": {},
                                                  "other_args": {}}
    assert info["window3"] == {"type": "sphere", "len_args": {"R": 60.0}, "los_args": {}, "other_args": {}}
