"""Host-side task logic on the CPU: the public task classes run end to end
(SFCProjection -> Corr_2PCF / Corr_3PCF_Multipole) with their GPU kernels
replaced by the float64 oracle (deposit, Parseval pair products, DDD_l,
mixing solve), against reference goldens made with a random catalogue
(random = a projected field, so dr / rd / rr and delta = D - R take the
field paths).  Relative 1e-5 of the largest |value| (the fields are float32,
as on the GPU)."""
import os

import numpy as np
import pytest
import torch

import oracle
from pyhermes_gb300 import corr2pcf, kernels
from pyhermes_gb300 import multipole as mp
from pyhermes_gb300.phi import sample_scaling_function
from pyhermes_gb300.projection import SFCProjection

PHI = sample_scaling_function()


def _rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.fixture
def oracle_kernels(monkeypatch):
    def deposit(pos, w, J, box, phi, phi_res=1024, out_dtype=torch.float32, counts=False, workspace=None, out=None):
        eps = oracle.deposit(pos.cpu().numpy(), w.cpu().numpy(), phi.cpu().numpy(), J, box, phi_res)
        return torch.as_tensor(eps, dtype=out_dtype), None, None

    def rfft_field(eps):  # the "spectrum" handed to pair_products is the real field itself
        return eps.detach().double().cpu().clone()

    def pair_products(spectra, pairs, windows, exclude_k0=True, descs=None):
        from pyhermes_gb300.window import WIN_ARGS

        L = windows[0].L
        P = oracle.fourier_power(PHI, windows[0].bandwidth, L)
        if descs is not None:  # a window family: the template with each bin's lengths
            t = windows[0]
            specs = [{nm: d.len[j] * t.box_size / L for j, nm in enumerate(WIN_ARGS[t.type])} for d in descs]
            windows = [t] * len(descs)
        else:
            specs = [w.len_args for w in windows]
        vals, k0 = np.zeros((len(windows), len(pairs))), np.zeros(len(windows))
        for b, w in enumerate(windows):
            K = oracle.window_kernel(w.type, specs[b], L, P, mode=w.resolved_mode(), box=w.box_size)
            k0[b] = K[0, 0, 0]
            for c, (i, j) in enumerate(pairs):
                ei, ej = spectra[i].numpy(), spectra[j].numpy()
                vals[b, c] = oracle.pair_product(ei, ej, K)
                if exclude_k0:
                    vals[b, c] -= K[0, 0, 0] * ei.sum() * ej.sum() / float(L) ** 6
        return vals, k0

    class Engine:
        def __init__(self, eps1, eps2, eps3, phi_array, J, box_size, phi_resolution=1024, share23=None,
                     engine="tensor"):
            self.e = [e.double().cpu().numpy() for e in (eps1, eps2, eps3)]
            self.phi, self.box, self.res = phi_array, box_size, phi_resolution
            self.timing = {"fields_s": 0.0, "contract_s": 0.0}

        def ddd(self, pairs, l_min, l_max):
            return np.array([oracle.calc_ddd_multipole(*self.e, a, b, l_min, l_max, self.phi, self.res, self.box)[1]
                             for a, b in pairs])

        ddd_plain = ddd

    def mixing_solve(A, B, lmax, device="cuda"):
        sol = [oracle.solve_multipoles_from_ratio(a, b, lmax) for a, b in zip(np.atleast_2d(A), np.atleast_2d(B))]
        return tuple(np.array([s[k] for s in sol]) for k in range(3))

    monkeypatch.setattr(kernels, "deposit", deposit)
    monkeypatch.setattr(kernels, "deposit_rejected", lambda ws, device=None: 0)
    monkeypatch.setattr(corr2pcf, "rfft_field", rfft_field)
    monkeypatch.setattr(corr2pcf, "pair_products", pair_products)
    monkeypatch.setattr(mp, "MultipoleEngine", Engine)
    monkeypatch.setattr(mp, "mixing_solve", mixing_solve)


def _fields(g):
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                         "box_size": 1000.0}}, device="cpu").run(save_result=False)
    r = SFCProjection({"SFCProjection": {"particle_pos": g["rpos"], "J": 4, "box_size": 1000.0}},
                      device="cpu").run(save_result=False)
    return f, r


def test_corr2pcf_random_field_matches_reference(golden_dir, oracle_kernels):
    g = np.load(os.path.join(golden_dir, "random_catalogue_J4.npz"))
    f, r = _fields(g)
    d = corr2pcf.Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": r,
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"},
        "sampling": {"s": {"min": 100.0, "max": 300.0, "n": 3}},
        "products": ["dd", "dr", "rd", "rr", "delta_dd", "xi"]}}, device="cpu").run(save_result=False)
    for k in ("dd", "dr", "rd", "rr", "delta_dd", "xi"):
        assert _rel(getattr(d, k), g["r2_" + k]) < 1e-5, (k, getattr(d, k), g["r2_" + k])


def test_multipole_random_field_matches_reference(golden_dir, oracle_kernels):
    g = np.load(os.path.join(golden_dir, "random_catalogue_J4.npz"))
    f, r = _fields(g)
    d = mp.Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field": f, "random": r,
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [150.0, 200.0], "r13": [250.0, 300.0]},
        "l_min": 0, "l_max": 2, "summation_backend": "gb300",
        "products": ["ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"]}}, device="cpu").run(save_result=False)
    for k in ("ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"):
        assert _rel(getattr(d, k), g["r3_" + k]) < 1e-5, (k, getattr(d, k), g["r3_" + k])


def _cpu_triplet_sum(eps1, eps2, eps3, J, centers, offsets, phi_t, center_w=None, rho1=0.0, samples=False,
                     locality=True):
    """sum_i w_i n1_i sum_r n2 n3 with the oracle's float64 interpolation."""
    c = centers.double().cpu().numpy()
    phi = phi_t.double().cpu().numpy()
    e2, e3 = (e.double().cpu().numpy() for e in (eps2, eps3))
    n1 = oracle.interp(c, eps1.double().cpu().numpy(), phi, J) if eps1 is not None else rho1
    w = np.ones(c.shape[0]) if center_w is None else np.asarray(center_w, dtype=np.float64)
    total = 0.0
    for o in np.asarray(offsets, dtype=np.float64):
        total += float(np.sum(w * n1 * oracle.interp(c, e2, phi, J, offset=o[0:3])
                              * oracle.interp(c, e3, phi, J, offset=o[3:6])))
    return total, None


@pytest.mark.parametrize("case", ["fields", "uni1"])
def test_mc3pcf_random_fields_match_reference(golden_dir, oracle_kernels, monkeypatch, case):
    """Box-random MC 3PCF with random catalogues as fields: three random
    fields (rrr by Monte Carlo over the same centres and rotations), and a
    uniform vertex 1 with random fields 2 and 3 (rrr = rho1 RR23(r23))."""
    from pyhermes_gb300 import mc3pcf

    monkeypatch.setattr(mc3pcf, "triplet_sum", _cpu_triplet_sum)
    g = np.load(os.path.join(golden_dir, "mc3pcf_randoms_J4.npz"))
    f, r = _fields(g)
    params = {"sfc_field": f, "r12": 150.0, "r13": 250.0, "angle_param": "mu",
              "mu": {"mu_min": -0.8, "mu_max": 0.8, "n_mu": 3}, "n_rot": 3, "center": "box_random",
              "n_box_centers": 600, "base_seed": 42}
    if case == "fields":
        params.update(random=r, products=["zeta", "ddd"])
        keys = ("ddd", "delta_ddd", "rrr", "zeta")
    else:
        params.update(random1="uniform", random2=r, random3=r, products=["zeta"])
        keys = ("delta_ddd", "rrr", "zeta")
    d = mc3pcf.Corr_3PCF({"Corr_3PCF": params}, device="cpu").run()
    for k in keys:
        assert _rel(getattr(d, k), g[f"{case}_{k}"]) < 1e-5, (k, getattr(d, k), g[f"{case}_{k}"])


@pytest.mark.parametrize("mode", ["raw", "field", "unit"])
def test_task_weight_normalization_matches_reference(golden_dir, oracle_kernels, monkeypatch, mode):
    """Task-level weight_normalization on a catalogue field with field
    values: Corr_2PCF products and Counting densities for each mode, and the
    multipole task for 'field', against the reference golden."""
    from pyhermes_gb300 import mc3pcf
    from pyhermes_gb300.counting import Counting

    def interp(grid, J, scaled_pos, phi_t, offset=(0.0, 0.0, 0.0)):
        p = scaled_pos.cpu().numpy() if isinstance(scaled_pos, torch.Tensor) else np.asarray(scaled_pos)
        return torch.as_tensor(oracle.interp(p, grid.double().cpu().numpy(), phi_t.double().cpu().numpy(), J,
                                             offset=offset))

    monkeypatch.setattr(mc3pcf, "interp", interp)
    g = np.load(os.path.join(golden_dir, "normalization_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"],
                                         "field_value": g["field_value"], "J": 4, "box_size": 1000.0}},
                      device="cpu").run(save_result=False)
    d = corr2pcf.Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform", "weight_normalization": mode,
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"},
        "sampling": {"s": {"min": 100.0, "max": 300.0, "n": 3}},
        "products": ["dd", "rr", "delta_dd", "xi"]}}, device="cpu").run(save_result=False)
    for k in ("dd", "rr", "delta_dd", "xi"):
        assert _rel(getattr(d, k), g[f"n2_{mode}_{k}"]) < 1e-5, (mode, k, getattr(d, k), g[f"n2_{mode}_{k}"])
    c = Counting({"Counting": {"sfc_field": f, "random_count": 400, "seed": 5, "weight_normalization": mode}},
                 device="cpu").run(save_result=False)
    assert _rel(c.nx, g[f"count_{mode}_nx"]) < 1e-5, (mode, c.nx[:4], g[f"count_{mode}_nx"][:4])
    if mode == "field":
        d = mp.Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
            "sfc_field": f, "random": "uniform", "weight_normalization": "field",
            "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
            "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
            "sampling": {"mode": "paired", "r12": [150.0], "r13": [250.0]},
            "l_min": 0, "l_max": 1, "products": ["ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"]}},
            device="cpu").run(save_result=False)
        for k in ("ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"):
            assert _rel(getattr(d, k), g["n3_field_" + k]) < 1e-5, (k, getattr(d, k), g["n3_field_" + k])


def test_cross_fields_and_vertex_windows_match_reference(golden_dir, oracle_kernels, monkeypatch):
    """Distinct fields per vertex and per-vertex smoothing windows (field @ W
    by the oracle's kernel and FFT convolution): Corr_2PCF with
    sfc_field1 != sfc_field2 and window1, Corr_3PCF_Multipole with fields
    A, B, A, window2, grid sampling and l_min = 1."""
    from pyhermes_gb300 import window as win_mod

    def apply_window(eps, w, out=None):
        L = w.L
        K = oracle.window_kernel(w.type, w.len_args, L, oracle.fourier_power(PHI, w.bandwidth, L),
                                 mode=w.resolved_mode(), box=w.box_size)
        return torch.as_tensor(oracle.convolve(eps.double().cpu().numpy(), K), dtype=torch.float32)

    def as_array(w):
        return oracle.window_kernel(w.type, w.len_args, w.L, oracle.fourier_power(PHI, w.bandwidth, w.L),
                                    mode=w.resolved_mode(), box=w.box_size)

    monkeypatch.setattr(win_mod, "apply_window", apply_window)
    monkeypatch.setattr(win_mod.WindowFunc, "as_array", as_array)
    g = np.load(os.path.join(golden_dir, "cross_J4.npz"))
    a = SFCProjection({"SFCProjection": {"particle_pos": g["pa"], "catalog_weight": g["wa"], "J": 4,
                                         "box_size": 1000.0}}, device="cpu").run(save_result=False)
    b = SFCProjection({"SFCProjection": {"particle_pos": g["pb"], "J": 4, "box_size": 1000.0}},
                      device="cpu").run(save_result=False)
    d = corr2pcf.Corr_2PCF({"Corr_2PCF": {
        "sfc_field1": a, "sfc_field2": b, "random": "uniform",
        "window1": {"type": "gaussian", "len_args": {"R": 30.0}},
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"},
        "sampling": {"s": {"min": 100.0, "max": 300.0, "n": 3}},
        "products": ["dd", "delta_dd", "xi"]}}, device="cpu").run(save_result=False)
    for k in ("dd", "delta_dd", "rr", "xi"):
        assert _rel(getattr(d, k), g["c2_" + k]) < 1e-5, (k, getattr(d, k), g["c2_" + k])
    d = mp.Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field1": a, "sfc_field2": b, "sfc_field3": a, "random": "uniform",
        "window2": {"type": "gaussian", "len_args": {"R": 40.0}},
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "grid", "r12": [150.0, 200.0], "r13": [250.0]},
        "l_min": 1, "l_max": 2, "products": ["ddd_l", "delta_ddd_l"]}}, device="cpu").run(save_result=False)
    for k in ("ddd_l", "delta_ddd_l"):
        assert _rel(getattr(d, k), g["c3_" + k]) < 1e-5, (k, getattr(d, k), g["c3_" + k])


@pytest.mark.parametrize("kind", ["ring", "cylshell"])
def test_corr2pcf_rppi_sampling_matches_reference(golden_dir, oracle_kernels, kind):
    """(r_p, pi) sampling through the rppi_to_RH mapping (R = r_p, H = pi)."""
    g = np.load(os.path.join(golden_dir, "rppi_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                         "box_size": 1000.0}}, device="cpu").run(save_result=False)
    d = corr2pcf.Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform", "binning_window": {"type": kind, "mapping": "rppi_to_RH"},
        "sampling": {"rp": {"min": 60.0, "max": 180.0, "n": 3}, "pi": {"min": 30.0, "max": 90.0, "n": 2}},
        "products": ["delta_dd", "xi"]}}, device="cpu").run(save_result=False)
    assert d.xi.shape == (3, 2)
    for k in ("delta_dd", "xi"):
        assert _rel(getattr(d, k), g[f"{kind}_{k}"]) < 1e-5, (k, getattr(d, k), g[f"{kind}_{k}"])


@pytest.mark.parametrize("case", ["spec", "list"])
def test_mc3pcf_theta_sampling_matches_reference(golden_dir, oracle_kernels, monkeypatch, case):
    from pyhermes_gb300 import mc3pcf

    monkeypatch.setattr(mc3pcf, "triplet_sum", _cpu_triplet_sum)
    g = np.load(os.path.join(golden_dir, "mc_theta_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "J": 4, "box_size": 1000.0}},
                      device="cpu").run(save_result=False)
    theta = {"spec": {"theta_min": 0.3, "theta_max": 2.5, "n_theta": 3}, "list": [0.5, 1.5]}[case]
    d = mc3pcf.Corr_3PCF({"Corr_3PCF": {
        "sfc_field": f, "random": "uniform", "r12": 150.0, "r13": 250.0, "angle_param": "theta", "theta": theta,
        "n_rot": 3, "center": "box_random", "n_box_centers": 400, "base_seed": 11,
        "products": ["ddd", "rrr", "delta_ddd"]}}, device="cpu").run()
    for k in ("theta", "mu", "r23"):
        np.testing.assert_allclose(getattr(d, k), g[f"{case}_{k}"], rtol=1e-14, atol=1e-14)
    for k in ("ddd", "rrr", "delta_ddd", "xi23"):
        assert _rel(getattr(d, k), g[f"{case}_{k}"]) < 1e-5, (k, getattr(d, k), g[f"{case}_{k}"])


def test_pair_product_at_sample_matches_reference(golden_dir, oracle_kernels):
    """compute_pair_product_at_sample and Corr_2PCF.calc_pair_product
    (theory/corr2pcf.py:375-382, 632-645) in grid units, a scalar vertex
    included."""
    g = np.load(os.path.join(golden_dir, "pair_at_sample_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "J": 4, "box_size": 1000.0}},
                      device="cpu").run(save_result=False)
    bw = {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"}
    v1 = corr2pcf.compute_pair_product_at_sample({"s": 150.0}, f, None, bw)
    task = corr2pcf.Corr_2PCF({"Corr_2PCF": {"sfc_field": f, "binning_window": bw, "sampling": {"s": [150.0]}}},
                              device="cpu")
    v2 = task.calc_pair_product({"s": 220.0}, f)
    v3 = task.calc_pair_product({"s": 220.0}, f, 2.5e-4)
    np.testing.assert_allclose([v1, v2, v3], g["values"], rtol=1e-5)
