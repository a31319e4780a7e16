"""Generates the golden fixtures in tests/golden/ by running the UNMODIFIED
PyHermes reference (read from a local checkout) under a minimal stub package
(``tests/golden/refshim``: numba -> plain Python, PyWavelets ->
scaling-function cascade, termcolor/json5/yaml stubs).

Usage:  python tests/golden/make_golden.py /path/to/PyHermes [section ...]

Fixtures are small (J <= 5) seeded cases.  The tests never import the
reference; they read these .npz files.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _setup(ref_root):
    sys.path[:0] = [os.path.join(HERE, "refshim"), ref_root, REPO]
    import logging

    logging.disable(logging.CRITICAL)


def _save(name, **arrays):
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **arrays)
    print("wrote", path, {k: getattr(v, "shape", None) for k, v in arrays.items()})


def gen_phi():
    from pyhermes.utils.corr3pcf_multipoles import cal_gamma
    from pyhermes.utils.wavelet_grid import fourier_power_spectrum, sample_scaling_function

    phi = sample_scaling_function("db2", 10)
    pw16 = fourier_power_spectrum(phi, 0, 1, 16, 1024)
    pw32_bw2 = fourier_power_spectrum(phi, 0, 2, 64, 1024)
    gamma = cal_gamma(phi, 3, 1024)
    _save("phi_db2", phi=phi, power_L16=pw16, power_L32_bw2=pw32_bw2, gamma=gamma)


def _projection(pos, J, weights=None, field_value=None, mode="catalog", box=1000.0):
    from pyhermes.base.sfc_projection import SFCProjection

    params = {"particle_pos": pos, "J": J, "box_size": box, "weight_normalization": mode}
    if weights is not None:
        params["catalog_weight"] = weights
    if field_value is not None:
        params["field_value"] = field_value
    task = SFCProjection({"SFCProjection": params})
    return task.run(save_result=False)


def gen_deposit():
    rng = np.random.default_rng(0)
    cases = {}
    # uniform, unit weights, catalog normalisation (the CPU-runnable config at small J)
    pos = rng.uniform(0.0, 1000.0, (2000, 3))
    f = _projection(pos, 4)
    cases["uniform_J4"] = (pos, np.ones(2000), np.ones(2000), "catalog", 4, f)
    # weighted + field values, 'field' normalisation, J=5, includes exact cell edges
    pos = rng.uniform(0.0, 1000.0, (3000, 3))
    pos[:10] = np.floor(pos[:10] / (1000.0 / 32)) * (1000.0 / 32)  # exactly on cell corners
    pos[10:20, 0] = 0.0
    pos[20:30, 1] = np.nextafter(1000.0, 0.0)
    w = rng.lognormal(0.0, 0.3, 3000)
    q = rng.uniform(0.5, 1.5, 3000)
    f = _projection(pos, 5, weights=w, field_value=q, mode="field")
    cases["weighted_J5"] = (pos, w, q, "field", 5, f)
    # raw normalisation, single particle
    pos = np.array([[123.456, 987.654, 0.001]])
    f = _projection(pos, 4, weights=np.array([2.5]), mode="raw")
    cases["single_raw_J4"] = (pos, np.array([2.5]), np.ones(1), "raw", 4, f)
    for name, (pos, w, q, mode, J, f) in cases.items():
        _save(f"deposit_{name}", pos=pos, catalog_weight=w, field_value=q, mode=np.array(mode),
              J=np.array(J), box=np.array(1000.0), epsilon=f.epsilon,
              field_integral=np.array(f.sfc_info["field_integral"]),
              catalog_weight_sum=np.array(f.sfc_info["catalog_weight_sum"]),
              raw_field_weighted_sum=np.array(f.sfc_info["raw_field_weighted_sum"]))


WINDOW_CASES = {
    # name: (win_params, bandwidth)
    "sphere": ({"type": "sphere", "len_args": {"R": 90.0}}, 1),
    "gaussian": ({"type": "gaussian", "len_args": {"R": 70.0}}, 1),
    "shell": ({"type": "shell", "len_args": {"R": 150.0}}, 1),
    "thick_shell": ({"type": "thick_shell", "len_args": {"R": 120.0, "delta_R": 40.0}}, 1),
    "thick_shell_inner0": ({"type": "thick_shell", "len_args": {"R": 10.0, "delta_R": 40.0}}, 1),
    "gaussian_shell": ({"type": "gaussian_shell", "len_args": {"R_shell": 100.0, "R_smooth": 30.0}}, 1),
    "cubic": ({"type": "cubic", "len_args": {"Lx": 80.0, "Ly": 120.0, "Lz": 200.0}}, 1),
    "ring_z": ({"type": "ring", "len_args": {"R": 100.0, "H": 60.0}}, 1),
    "disk_z": ({"type": "disk", "len_args": {"R": 100.0, "H": 60.0}}, 1),
    "cylshell_z": ({"type": "cylshell", "len_args": {"R": 100.0, "H": 60.0}}, 1),
    "cylinder_z": ({"type": "cylinder", "len_args": {"R": 100.0, "H": 60.0}}, 1),
    "ring_tilted": ({"type": "ring", "len_args": {"R": 100.0, "H": 60.0},
                     "los_args": {"nx": 1.0, "ny": 2.0, "nz": 2.0}}, 1),
    "cw": ({"type": "cw", "len_args": {"R": 60.0}}, 1),
    "cws": ({"type": "cws", "len_args": {"R": 60.0}}, 1),
    "gdw": ({"type": "gdw", "len_args": {"R": 60.0}}, 1),
    "dirderiv": ({"type": "directional_derivative", "los_args": {"nx": 0.0, "ny": 1.0, "nz": 1.0}}, 1),
    "laplacian": ({"type": "laplacian"}, 1),
    "inverse_laplacian": ({"type": "inverse_laplacian"}, 1),
    "gaussian_bw2": ({"type": "gaussian", "len_args": {"R": 40.0}}, 2),
}


def _sfc_params(J):
    return {"J": J, "box_size": 1000.0, "phi_resolution": 1024, "wavelet_mode": "db2", "wavelet_level": 10}


def gen_windows():
    from pyhermes.io.window import WindowFunc

    out = {}
    for name, (wp, bw) in WINDOW_CASES.items():
        w = WindowFunc(dict(wp), _sfc_params(4), bandwidth=bw)
        out[name] = np.asarray(w.as_array())
    _save("windows_J4", **out)


def gen_convolution():
    from pyhermes.io.window import WindowFunc

    rng = np.random.default_rng(7)
    pos = rng.uniform(0.0, 1000.0, (4000, 3))
    f = _projection(pos, 5, weights=rng.lognormal(0.0, 0.3, 4000))
    res = {"pos": pos, "epsilon": f.epsilon}
    for name in ("gaussian", "thick_shell", "ring_tilted", "dirderiv", "inverse_laplacian"):
        w = WindowFunc(dict(WINDOW_CASES[name][0]), f.sfc_info)
        res["conv_" + name] = (f @ w).epsilon
    _save("convolution_J5", **res)


def gen_corr2pcf():
    from pyhermes.theory.corr2pcf import Corr_2PCF

    rng = np.random.default_rng(11)
    pos = rng.uniform(0.0, 1000.0, (6000, 3))
    pos[:2000] = (pos[:2000] * 0.25 + 300.0)  # a clump so xi is not pure noise
    w = rng.lognormal(0.0, 0.3, 6000)
    f = _projection(pos, 5, weights=w)
    out = {"pos": pos, "weights": w}
    task = Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform",
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": 40.0},
                           "mapping": "s_to_R"},
        "sampling": {"s": {"min": 60.0, "max": 300.0, "n": 5}},
        "products": ["dd", "dr", "delta_dd", "rr", "xi"]}})
    d = task.run(save_result=False)
    for k in ("dd", "dr", "delta_dd", "rr", "xi"):
        out["iso_" + k] = np.asarray(getattr(d, k))
    task = Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform",
        "binning_window": {"type": "ring"},
        "sampling": {"s": {"min": 80.0, "max": 240.0, "n": 3}, "mu": {"min": 0.1, "max": 0.9, "n": 3}},
        "products": ["delta_dd", "xi"]}})
    d = task.run(save_result=False)
    out["smu_delta_dd"] = np.asarray(d.delta_dd)
    out["smu_xi"] = np.asarray(d.xi)
    task = Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform", "window": {"type": "gaussian", "len_args": {"R": 40.0}},
        "binning_window": {"type": "shell", "len_args": ["R"], "mapping": "s_to_R"},
        "sampling": {"s": {"min": 80.0, "max": 200.0, "n": 3}},
        "products": ["xi"]}})
    d = task.run(save_result=False)
    out["smooth_xi"] = np.asarray(d.xi)
    out["smooth_delta_dd"] = np.asarray(d.delta_dd)
    _save("corr2pcf_J5", **out)


def gen_multipole():
    from pyhermes.theory.corr3pcf_multipole import Corr_3PCF_Multipole
    from pyhermes.utils.radial_multipole_windows import calculate_radial_multipole_window_array
    from pyhermes.utils.special_functions import spherical_harmonic_numba, spherical_jn_numba
    from pyhermes.utils.wavelet_grid import fourier_power_spectrum

    out = {}
    # special functions on a grid of arguments
    xs = np.array([0.0, 1e-3, 0.04, 0.3, 1.0, 2.5, 7.0, 12.0, 33.0, 80.0])
    out["jn"] = np.array([[spherical_jn_numba(l, x) for x in xs] for l in range(11)])
    out["jn_x"] = xs
    ks = np.array([[0.1, 0.2, 0.3], [-0.4, 0.1, -0.2], [0.0, 0.0, 0.5], [0.3, -0.3, 0.0], [-0.1, -0.2, -0.3]])
    out["ylm"] = np.array([[[spherical_harmonic_numba(l, m, *k) for k in ks] for m in range(-l, l + 1)]
                           + [[0j] * len(ks)] * (10 - 2 * l) for l in range(5)])
    out["ylm_k"] = ks
    phi = np.load(os.path.join(HERE, "phi_db2.npz"))["phi"]
    P = fourier_power_spectrum(phi, 0, 1, 16, 1024)
    for (l, m) in [(0, 0), (2, 1), (3, -2), (4, 4)]:
        out[f"window_l{l}_m{m}"] = calculate_radial_multipole_window_array(
            16, P, {"R": 180.0}, "shell", l, m, box_size=1000.0)
    # the task: J=4, clustered catalogue, two (r12, r13) samples, l <= 2
    rng = np.random.default_rng(21)
    pos = rng.uniform(0.0, 1000.0, (3000, 3))
    pos[:1200] = pos[:1200] * 0.3 + 350.0
    w = rng.lognormal(0.0, 0.3, 3000)
    f = _projection(pos, 4, weights=w)
    task = Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field": f, "random": "uniform",
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [150.0, 200.0], "r13": [250.0, 300.0]},
        "l_min": 0, "l_max": 2, "summation_backend": "cpu", "products": ["ddd_l", "zeta_l"]}})
    d = task.run(save_result=False)
    out.update({"pos": pos, "weights": w, "epsilon": f.epsilon, "l": d.l, "ddd_l": d.ddd_l,
                "delta_ddd_l": d.delta_ddd_l, "rrr_l": d.rrr_l, "zeta_l": d.zeta_l,
                "zeta_condition": d.zeta_condition})
    _save("multipole_J4", **out)


def gen_mc3pcf():
    from pyhermes.theory.corr3pcf import Corr_3PCF
    from pyhermes.utils.corr3pcf_kernels import generate_triangle_offsets

    rng = np.random.default_rng(31)
    pos = rng.uniform(0.0, 1000.0, (4000, 3))
    pos[:1500] = pos[:1500] * 0.3 + 300.0
    w = rng.lognormal(0.0, 0.3, 4000)
    f = _projection(pos, 4, weights=w)
    out = {"pos": pos, "weights": w}
    offs = [generate_triangle_offsets(2.0, 3.5, m, p, c, a)
            for m, p, c, a in [(0.3, 1.0, 0.2, 2.0), (-0.7, 4.0, -0.9, 0.5), (0.999, 0.1, 0.9999, 6.0)]]
    out["offsets"] = np.array(offs)
    task = Corr_3PCF({"Corr_3PCF": {
        "sfc_field": f, "random": "uniform", "r12": 150.0, "r13": 250.0, "angle_param": "mu",
        "mu": {"mu_min": -0.8, "mu_max": 0.8, "n_mu": 3}, "n_rot": 3, "center": "box_random",
        "n_box_centers": 600, "base_seed": 42, "products": ["Q", "ddd"]}})
    d = task.run(save_result=False)
    for k in ("mu", "ddd", "rrr", "delta_ddd", "xi12", "xi13", "xi23", "zeta", "zeta_H", "Q"):
        out["box_" + k] = np.asarray(getattr(d, k))
    _save("mc3pcf_J4", **out)


def gen_mc3pcf_particle():
    """center='particle': data-particle centres for ddd / d_delta_dd, explicit
    random centres (random_pos1) or the uniform-random shortcut for
    r_delta_dd, delta_ddd = d_delta_dd - r_delta_dd (corr3pcf.py:1134-1180,
    1590-1614)."""
    from pyhermes.theory.corr3pcf import Corr_3PCF

    rng = np.random.default_rng(41)
    pos = rng.uniform(0.0, 1000.0, (3000, 3))
    pos[:1000] = pos[:1000] * 0.3 + 300.0
    w = rng.lognormal(0.0, 0.3, 3000)
    f = _projection(pos, 4, weights=w)
    cpos = pos[::5].copy()
    cw = w[::5].copy()
    rpos = rng.uniform(0.0, 1000.0, (500, 3))
    rw = rng.uniform(0.5, 1.5, 500)
    out = {"pos": pos, "weights": w, "cpos": cpos, "cw": cw, "rpos": rpos, "rw": rw,
           "epsilon": np.asarray(f.epsilon), "field_integral": float(f.sfc_info["field_integral"])}
    common = {"sfc_field": f, "random": "uniform", "r12": 150.0, "r13": 250.0, "angle_param": "mu",
              "mu": {"mu_min": -0.8, "mu_max": 0.8, "n_mu": 3}, "n_rot": 3, "center": "particle",
              "base_seed": 7, "particle_pos1": cpos, "particle_weight1": cw}
    d = Corr_3PCF({"Corr_3PCF": dict(common, random_pos1=rpos, random_weight1=rw,
                                     products=["ddd", "rrr", "d_delta_dd", "r_delta_dd", "delta_ddd"])}).run(
        save_result=False)
    for k in ("mu", "ddd", "rrr", "d_delta_dd", "r_delta_dd", "delta_ddd"):
        out["rpos_" + k] = np.asarray(getattr(d, k))
    d = Corr_3PCF({"Corr_3PCF": dict(common, products=["zeta", "ddd"])}).run(save_result=False)
    for k in ("ddd", "rrr", "d_delta_dd", "r_delta_dd", "delta_ddd", "xi23", "zeta"):
        out["uni_" + k] = np.asarray(getattr(d, k))
    # smoothing windows: a shared one and a vertex-3 override (theory/corr3pcf.py:176-183, 1038-1104)
    d = Corr_3PCF({"Corr_3PCF": dict(common, window={"type": "gaussian", "len_args": {"R": 40.0}},
                                     window3={"type": "sphere", "len_args": {"R": 60.0}},
                                     products=["zeta", "ddd"])}).run(save_result=False)
    for k in ("ddd", "rrr", "d_delta_dd", "r_delta_dd", "delta_ddd", "xi23", "zeta"):
        out["win_" + k] = np.asarray(getattr(d, k))
    _save("mc3pcf_particle_J4", **out)


def gen_random_catalogue():
    """Data and random catalogues (random = a projected field, not
    'uniform'): Corr_2PCF dd/dr/rd/rr/delta_dd/xi with thick shells and
    Corr_3PCF_Multipole ddd_l/delta_ddd_l/rrr_l/zeta_l with delta = D - R."""
    from pyhermes.theory.corr2pcf import Corr_2PCF
    from pyhermes.theory.corr3pcf_multipole import Corr_3PCF_Multipole

    rng = np.random.default_rng(51)
    pos = rng.uniform(0.0, 1000.0, (3000, 3))
    pos[:1200] = pos[:1200] * 0.3 + 350.0
    w = rng.lognormal(0.0, 0.3, 3000)
    rpos = rng.uniform(0.0, 1000.0, (9000, 3))
    f = _projection(pos, 4, weights=w)
    r = _projection(rpos, 4)
    out = {"pos": pos, "weights": w, "rpos": rpos}
    d = Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": r,
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"},
        "sampling": {"s": {"min": 100.0, "max": 300.0, "n": 3}},
        "products": ["dd", "dr", "rd", "rr", "delta_dd", "xi"]}}).run(save_result=False)
    for k in ("dd", "dr", "rd", "rr", "delta_dd", "xi"):
        out["r2_" + k] = np.asarray(getattr(d, k))
    d = Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field": f, "random": r,
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [150.0, 200.0], "r13": [250.0, 300.0]},
        "l_min": 0, "l_max": 2, "summation_backend": "cpu",
        "products": ["ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"]}}).run(save_result=False)
    for k in ("ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"):
        out["r3_" + k] = np.asarray(getattr(d, k))
    _save("random_catalogue_J4", **out)


def gen_mc3pcf_randoms():
    """Box-random MC 3PCF with random catalogues as fields: three random
    fields (rrr by Monte Carlo) and a uniform random vertex 1 with random
    fields 2 and 3 (rrr = rho1 RR23(r23))."""
    from pyhermes.theory.corr3pcf import Corr_3PCF

    rng = np.random.default_rng(61)
    pos = rng.uniform(0.0, 1000.0, (3000, 3))
    pos[:1200] = pos[:1200] * 0.3 + 350.0
    w = rng.lognormal(0.0, 0.3, 3000)
    rpos = rng.uniform(0.0, 1000.0, (9000, 3))
    f = _projection(pos, 4, weights=w)
    r = _projection(rpos, 4)
    out = {"pos": pos, "weights": w, "rpos": rpos}
    common = {"sfc_field": f, "r12": 150.0, "r13": 250.0, "angle_param": "mu",
              "mu": {"mu_min": -0.8, "mu_max": 0.8, "n_mu": 3}, "n_rot": 3, "center": "box_random",
              "n_box_centers": 600, "base_seed": 42}
    d = Corr_3PCF({"Corr_3PCF": dict(common, random=r, products=["zeta", "ddd"])}).run(save_result=False)
    for k in ("ddd", "delta_ddd", "rrr", "zeta"):
        out["fields_" + k] = np.asarray(getattr(d, k))
    d = Corr_3PCF({"Corr_3PCF": dict(common, random1="uniform", random2=r, random3=r, products=["zeta"])}).run(
        save_result=False)
    for k in ("delta_ddd", "rrr", "zeta"):
        out["uni1_" + k] = np.asarray(getattr(d, k))
    _save("mc3pcf_randoms_J4", **out)


def gen_normalization():
    """Task-level weight_normalization on a catalogue field with field values
    (io/sfc_field.py:32-38 modes; each task switches the field before use):
    Corr_2PCF and Counting for raw / field / unit, Corr_3PCF_Multipole for
    field."""
    from pyhermes.theory.corr2pcf import Corr_2PCF
    from pyhermes.theory.corr3pcf_multipole import Corr_3PCF_Multipole
    from pyhermes.theory.counting import Counting

    rng = np.random.default_rng(71)
    pos = rng.uniform(0.0, 1000.0, (3000, 3))
    pos[:1200] = pos[:1200] * 0.3 + 350.0
    w = rng.lognormal(0.0, 0.3, 3000)
    fv = rng.uniform(0.5, 2.0, 3000)
    f = _projection(pos, 4, weights=w, field_value=fv)
    out = {"pos": pos, "weights": w, "field_value": fv, "epsilon": np.asarray(f.epsilon),
           "field_integral": float(f.sfc_info["field_integral"])}
    for mode in ("raw", "field", "unit"):
        d = Corr_2PCF({"Corr_2PCF": {
            "sfc_field": f, "random": "uniform", "weight_normalization": mode,
            "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"},
            "sampling": {"s": {"min": 100.0, "max": 300.0, "n": 3}},
            "products": ["dd", "rr", "delta_dd", "xi"]}}).run(save_result=False)
        for k in ("dd", "rr", "delta_dd", "xi"):
            out[f"n2_{mode}_{k}"] = np.asarray(getattr(d, k))
        c = Counting({"Counting": {"sfc_field": f, "random_count": 400, "seed": 5,
                                   "weight_normalization": mode}}).run(save_result=False)
        out[f"count_{mode}_nx"] = np.asarray(c.nx)
    d = Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field": f, "random": "uniform", "weight_normalization": "field",
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [150.0], "r13": [250.0]},
        "l_min": 0, "l_max": 1, "summation_backend": "cpu",
        "products": ["ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"]}}).run(save_result=False)
    for k in ("ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"):
        out["n3_field_" + k] = np.asarray(getattr(d, k))
    _save("normalization_J4", **out)


def gen_cross():
    """Distinct fields per vertex and per-vertex smoothing windows:
    Corr_2PCF (sfc_field1 != sfc_field2, window1) and Corr_3PCF_Multipole
    (fields A, B, A, window2, grid sampling, l_min = 1)."""
    from pyhermes.theory.corr2pcf import Corr_2PCF
    from pyhermes.theory.corr3pcf_multipole import Corr_3PCF_Multipole

    rng = np.random.default_rng(81)
    pa = rng.uniform(0.0, 1000.0, (3000, 3))
    pa[:1200] = pa[:1200] * 0.3 + 350.0
    wa = rng.lognormal(0.0, 0.3, 3000)
    pb = rng.uniform(0.0, 1000.0, (2500, 3))
    pb[:800] = pb[:800] * 0.25 + 420.0
    a = _projection(pa, 4, weights=wa)
    b = _projection(pb, 4)
    out = {"pa": pa, "wa": wa, "pb": pb}
    d = Corr_2PCF({"Corr_2PCF": {
        "sfc_field1": a, "sfc_field2": b, "random": "uniform",
        "window1": {"type": "gaussian", "len_args": {"R": 30.0}},
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"},
        "sampling": {"s": {"min": 100.0, "max": 300.0, "n": 3}},
        "products": ["dd", "delta_dd", "xi"]}}).run(save_result=False)
    for k in ("dd", "delta_dd", "rr", "xi"):
        out["c2_" + k] = np.asarray(getattr(d, k))
    d = Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field1": a, "sfc_field2": b, "sfc_field3": a, "random": "uniform",
        "window2": {"type": "gaussian", "len_args": {"R": 40.0}},
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "grid", "r12": [150.0, 200.0], "r13": [250.0]},
        "l_min": 1, "l_max": 2, "summation_backend": "cpu", "products": ["ddd_l", "delta_ddd_l"]}}).run(
        save_result=False)
    for k in ("ddd_l", "delta_ddd_l"):
        out["c3_" + k] = np.asarray(getattr(d, k))
    _save("cross_J4", **out)


def gen_io():
    """Files written by the reference's own save methods (NumPy-framed
    pickles, io/pickle_compat.py): a projected field (io/sfc_field.py:546)
    and the results of Corr_2PCF, Counting, Corr_3PCF and
    Corr_3PCF_Multipole (io/corr2pcf.py:90, io/counting.py:29,
    io/corr3pcf.py:55, io/corr3pcf_multipole.py:39)."""
    from pyhermes.theory.corr2pcf import Corr_2PCF
    from pyhermes.theory.corr3pcf import Corr_3PCF
    from pyhermes.theory.corr3pcf_multipole import Corr_3PCF_Multipole
    from pyhermes.theory.counting import Counting

    d_io = os.path.join(HERE, "io")
    os.makedirs(d_io, exist_ok=True)
    cwd = os.getcwd()
    os.chdir(d_io)  # the result files record fout_path; keep it relative
    rng = np.random.default_rng(91)
    pos = rng.uniform(0.0, 1000.0, (2000, 3))
    pos[:800] = pos[:800] * 0.3 + 350.0
    w = rng.lognormal(0.0, 0.3, 2000)
    np.savez_compressed("catalogue.npz", pos=pos, weights=w)
    f = _projection(pos, 4, weights=w)
    f.save_sfc_field("./field_J4.pkl", overwrite=True)
    Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform", "fout_path": "./corr2pcf_J4.pkl",
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"},
        "sampling": {"s": {"min": 100.0, "max": 300.0, "n": 3}}, "products": ["dd", "xi"]}}).run(
        save_result=True, overwrite=True)
    Counting({"Counting": {"sfc_field": f, "random_count": 50, "seed": 3,
                           "fout_path": "./counting_J4.pkl"}}).run(save_result=True, overwrite=True)
    Corr_3PCF({"Corr_3PCF": {
        "sfc_field": f, "random": "uniform", "r12": 150.0, "r13": 250.0, "angle_param": "mu",
        "mu": {"mu_min": -0.5, "mu_max": 0.5, "n_mu": 2}, "n_rot": 2, "center": "box_random",
        "n_box_centers": 100, "base_seed": 42, "products": ["zeta", "ddd"],
        "fout_path": "./corr3pcf_J4.pkl"}}).run(save_result=True, overwrite=True)
    Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field": f, "random": "uniform", "fout_path": "./corr3pcf_multipole_J4.pkl",
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [150.0], "r13": [250.0]},
        "l_min": 0, "l_max": 1, "summation_backend": "cpu", "products": ["ddd_l", "zeta_l"]}}).run(
        save_result=True, overwrite=True)
    os.chdir(cwd)
    print("wrote", sorted(os.listdir(d_io)))


def gen_rppi():
    """Corr_2PCF with (r_p, pi) sampling: ring and cylinder-shell bins
    through the rppi_to_RH mapping (theory/corr2pcf.py:287-296)."""
    from pyhermes.theory.corr2pcf import Corr_2PCF

    rng = np.random.default_rng(101)
    pos = rng.uniform(0.0, 1000.0, (3000, 3))
    pos[:1200] = pos[:1200] * 0.3 + 350.0
    w = rng.lognormal(0.0, 0.3, 3000)
    f = _projection(pos, 4, weights=w)
    out = {"pos": pos, "weights": w}
    for kind in ("ring", "cylshell"):
        d = Corr_2PCF({"Corr_2PCF": {
            "sfc_field": f, "random": "uniform",
            "binning_window": {"type": kind, "mapping": "rppi_to_RH"},
            "sampling": {"rp": {"min": 60.0, "max": 180.0, "n": 3}, "pi": {"min": 30.0, "max": 90.0, "n": 2}},
            "products": ["delta_dd", "xi"]}}).run(save_result=False)
        out[f"{kind}_delta_dd"] = np.asarray(d.delta_dd)
        out[f"{kind}_xi"] = np.asarray(d.xi)
    _save("rppi_J4", **out)


def _info_json(info):
    import json

    def clean(v):
        if isinstance(v, dict):
            return {k: clean(x) for k, x in v.items() if k not in ("phi_array",)}
        if isinstance(v, (list, tuple)):
            return [clean(x) for x in v]
        if isinstance(v, (np.floating, np.integer)):
            return v.item()
        if isinstance(v, np.ndarray):
            return v.tolist()
        return v

    return json.dumps(clean(info), sort_keys=True)


def gen_field_algebra():
    """SFCField algebra and normalisation (io/sfc_field.py:152-423, 484-530):
    the epsilon and sfc_info (without phi_array, as JSON) of each result,
    mean densities and field_density_at_pos options."""
    rng = np.random.default_rng(111)
    pa = rng.uniform(0.0, 1000.0, (2000, 3))
    pa[:800] = pa[:800] * 0.3 + 350.0
    wa = rng.lognormal(0.0, 0.3, 2000)
    fva = rng.uniform(0.5, 2.0, 2000)
    pb = rng.uniform(0.0, 1000.0, (1500, 3))
    a = _projection(pa, 4, weights=wa, field_value=fva)
    b = _projection(pb, 4)
    q = rng.uniform(0.0, 1000.0, (200, 3))
    out = {"pa": pa, "wa": wa, "fva": fva, "pb": pb, "query": q}
    results = {"add": a + b, "sub": a - b, "mul": a * b, "adds": a + 0.5, "subs": a - 0.25, "rsubs": 1.0 - a,
               "muls": 3.0 * a, "divs": a / 4.0, "switch_raw": a.switch_weight_normalization("raw"),
               "switch_field": a.switch_weight_normalization("field"), "unit": a.to_unit_weight(),
               "with_raw": a.with_normalization("raw")}
    for name, r in results.items():
        out[name + "_eps"] = np.asarray(r.epsilon)
        out[name + "_info"] = np.array(_info_json(r.sfc_info))
    dens = {}
    for norm in (None, "raw", "field", "unit"):
        for unit in ("grid", "physical"):
            key = f"{norm}_{unit}"
            dens["mean_" + key] = a.field_mean_density(normalization=norm, value_unit=unit)
            out["at_" + key] = np.asarray(a.field_density_at_pos(q, normalization=norm, value_unit=unit))
    out["means"] = np.array(_info_json(dens))
    _save("field_algebra_J4", **out)


def gen_particle_data():
    """SFCField.get_particle_data (io/sfc_field.py:425-482) from a saved
    particle dataset (base/sfc_projection.py:195-219)."""
    import tempfile

    from pyhermes.base.sfc_projection import SFCProjection

    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        rng = np.random.default_rng(131)
        pos = rng.uniform(0.0, 1000.0, (400, 3))
        g = SFCProjection({"SFCProjection": {"particle_pos": pos, "catalog_weight": rng.lognormal(0.0, 0.3, 400),
                                             "J": 4, "box_size": 1000.0, "save_particle_data": True,
                                             "particle_data_path": os.path.join(tmp, "p.npz")}}).run(
            save_result=False)
        out["saved_pos_in"] = pos
        for k, v in g.get_particle_data().items():
            out["saved__" + k] = np.asarray(v)
        with np.load(os.path.join(tmp, "p.npz")) as z:
            for k in z.files:
                out["savedfile__" + k] = z[k]
    _save("particle_data_J4", **out)


def gen_composite_windows():
    """WindowFunc composite algebra (io/window.py:345-485): kernels of
    window +, -, x with windows and scalars, and the file a composite saves."""
    import tempfile

    from pyhermes.io.sfc_field import read_numpy_pickle
    from pyhermes.io.window import WindowFunc

    sfc = _sfc_params(4)
    a = WindowFunc({"type": "gaussian", "len_args": {"R": 30.0}}, sfc)
    b = WindowFunc({"type": "sphere", "len_args": {"R": 50.0}}, sfc)
    out = {}
    for name, w in {"add": a + b, "sub": a - 0.5 * b, "neg": -a, "prod": a * b, "div": a / 4.0,
                    "nested": (a + b) * 2.0 - a}.items():
        out[name + "_kernel"] = np.asarray(w.as_array())
    with tempfile.TemporaryDirectory() as tmp:
        fn = os.path.join(tmp, "w.pkl")
        (a + b).save(fn)
        with open(fn, "rb") as f:
            d = read_numpy_pickle(f)
    out["saved_keys"] = np.array(list(d.keys()))
    out["saved_info"] = np.array(_info_json({k: v for k, v in d.items() if k != "window_kernal"}))
    out["saved_kernel"] = np.asarray(d["window_kernal"])
    _save("composite_windows_J4", **out)


def gen_custom_windows():
    """WindowFunc with a user callable (io/window.py:88-96, :274-332;
    utils/convolution.py): kernels in full_rfft (default), octant,
    complex_rfft and bandwidth 2, a scalar-only function, a callable named
    with a built-in type, and a field convolved with one of them."""
    from custom_window_funcs import aniso_gauss, odd_los, skewed_gauss, stepped_tophat
    from pyhermes.io.window import WindowFunc

    sfc = _sfc_params(4)
    cases = {
        "gauss_full": ({"func": aniso_gauss, "len_args": {"R": 60.0}}, 1),
        "gauss_octant": ({"func": aniso_gauss, "len_args": {"R": 60.0}, "other_args": {"q": 0.7},
                          "kernel_mode": "octant"}, 1),
        "gauss_bw2": ({"func": aniso_gauss, "len_args": {"R": 40.0}}, 2),
        "skew_full": ({"func": skewed_gauss, "len_args": {"R": 50.0}}, 1),
        "skew_octant": ({"func": skewed_gauss, "len_args": {"R": 50.0}, "kernel_mode": "octant"}, 1),
        "skew_auto_axis": ({"func": skewed_gauss, "len_args": {"R": 50.0}, "kernel_mode": "auto",
                            "los_args": [0.0, 0.0, 1.0]}, 1),
        "step_full": ({"func": stepped_tophat, "len_args": {"R": 80.0}}, 1),
        "odd_complex": ({"func": odd_los, "len_args": {"R": 50.0}, "los_args": {"nx": 0.0, "ny": 1.0, "nz": 1.0},
                         "kernel_mode": "complex_rfft"}, 1),
        "named_gaussian": ({"type": "gaussian", "func": aniso_gauss, "len_args": {"R": 60.0}}, 1),
    }
    out = {}
    for name, (wp, bw) in cases.items():
        w = WindowFunc(dict(wp), sfc, bandwidth=bw)
        out[name] = np.asarray(w.as_array())
        out[name + "_meta"] = np.array([w.type, w.kernel_mode])
    rng = np.random.default_rng(21)
    pos = rng.uniform(0.0, 1000.0, (3000, 3))
    wts = rng.lognormal(0.0, 0.3, 3000)
    f = _projection(pos, 4, weights=wts)
    out.update({"pos": pos, "weights": wts, "epsilon": f.epsilon})
    out["conv_skew"] = (f @ WindowFunc(dict(cases["skew_full"][0]), f.sfc_info)).epsilon
    # a uniform random behind windows with W(0) = 2 (theory/corr3pcf_multipole.py:607-619)
    from custom_window_funcs import doubled_gauss
    from pyhermes.theory.corr3pcf_multipole import Corr_3PCF_Multipole

    # a vertex window needs a 'type' to be taken (theory/corr3pcf_multipole.py:71-74)
    win = {"type": "custom", "func": doubled_gauss, "len_args": {"R": 40.0}}
    d = Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field": f, "random": "uniform", "window1": dict(win), "window2": dict(win), "window3": dict(win),
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [150.0, 200.0], "r13": [250.0, 300.0]},
        "l_min": 0, "l_max": 2, "summation_backend": "cpu",
        "products": ["ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"]}}).run(save_result=False)
    for k in ("ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"):
        out["mp_" + k] = np.asarray(getattr(d, k))
    # Corr_2PCF with a user-callable binning window (theory/corr2pcf.py:366-382)
    from custom_window_funcs import j0_shell
    from pyhermes.theory.corr2pcf import Corr_2PCF

    d = Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform",
        "binning_window": {"func": j0_shell, "len_args": {"R": None}, "mapping": "s_to_R"},
        "sampling": {"s": {"min": 100.0, "max": 300.0, "n": 3}},
        "products": ["dd", "delta_dd", "xi"]}}).run(save_result=False)
    for k in ("dd", "delta_dd", "rr", "xi"):
        out["c2_" + k] = np.asarray(getattr(d, k))
    _save("custom_windows_J4", **out)


def gen_full_fft_windows():
    """Complex full-FFT windows (io/window.py:198-264): legendre_multipole
    (utils/legendre_windows.py) and radial_multipole
    (utils/radial_multipole_windows.py:267-316) kernels, and a field
    convolved with them (utils/convolution.py:291-295)."""
    from pyhermes.io.window import WindowFunc

    cases = {
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
    rng = np.random.default_rng(33)
    pos = rng.uniform(0.0, 1000.0, (2500, 3))
    pos[:900] = pos[:900] * 0.3 + 300.0
    f = _projection(pos, 4)
    out = {"pos": pos, "epsilon": f.epsilon}
    for name, wp in cases.items():
        w = WindowFunc(dict(wp), f.sfc_info)
        out[name + "_kernel"] = np.asarray(w.as_array())
        out[name + "_conv"] = np.asarray((f @ w).epsilon)
    _save("full_fft_windows_J4", **out)


def gen_phi_at_pos():
    """SFCField.phi_at_pos (io/sfc_field.py:484-485,
    utils/wavelet_grid.py:121-140): coarse cells and 3x3x3 stencils."""
    rng = np.random.default_rng(44)
    pos = rng.uniform(0.0, 1000.0, (200, 3))
    pos[:5] = [[0.0, 0.0, 0.0], [999.999, 500.0, 62.5], [62.5, 125.0, 187.5], [1e-9, 999.0, 3.3], [500.0, 0.5, 0.0]]
    f = _projection(pos, 4)
    coarse, local = f.phi_at_pos(pos)
    _save("phi_at_pos_J4", pos=pos, coarse=coarse, local=local)


def gen_mc_theta():
    """Corr_3PCF with angle_param='theta' (a min/max/n spec and a list)."""
    from pyhermes.theory.corr3pcf import Corr_3PCF

    rng = np.random.default_rng(141)
    pos = rng.uniform(0.0, 1000.0, (3000, 3))
    pos[:1200] = pos[:1200] * 0.3 + 350.0
    f = _projection(pos, 4)
    out = {"pos": pos}
    for name, theta in {"spec": {"theta_min": 0.3, "theta_max": 2.5, "n_theta": 3}, "list": [0.5, 1.5]}.items():
        d = Corr_3PCF({"Corr_3PCF": {
            "sfc_field": f, "random": "uniform", "r12": 150.0, "r13": 250.0, "angle_param": "theta",
            "theta": theta, "n_rot": 3, "center": "box_random", "n_box_centers": 400, "base_seed": 11,
            "products": ["ddd", "rrr", "delta_ddd"]}}).run(save_result=False)
        for k in ("theta", "mu", "r23", "ddd", "rrr", "delta_ddd", "xi23"):
            out[f"{name}_{k}"] = np.asarray(getattr(d, k))
    _save("mc_theta_J4", **out)


def gen_counting():
    from pyhermes.io.window import WindowFunc
    from pyhermes.theory.counting import Counting

    rng = np.random.default_rng(17)
    pos = rng.uniform(0.0, 1000.0, (3000, 3))
    pos[:1000] = pos[:1000] * 0.25 + 400.0
    w = rng.lognormal(0.0, 0.3, 3000)
    f = _projection(pos, 4, weights=w)
    q = rng.uniform(0.0, 1000.0, (500, 3))
    win = WindowFunc({"type": "gaussian", "len_args": {"R": 80.0}}, f.sfc_info)
    d = Counting({"Counting": {"sfc_field": f, "random_count": 700, "seed": 5,
                               "window": {"type": "gaussian", "len_args": {"R": 80.0}}}}).run(save_result=False)
    _save("counting_J4", pos=pos, weights=w, query=q,
          nx_physical=f.field_density_at_pos(q, value_unit="physical"),
          nx_grid=f.field_density_at_pos(q, value_unit="grid"),
          nx_filter=f.field_density_at_pos(q, filter=win),
          nx_unit=f.field_density_at_pos(q, normalization="unit"),
          counting_nx=np.asarray(d.nx))


def gen_tabulated():
    from pyhermes.theory.corr3pcf_multipole import Corr_3PCF_Multipole
    from pyhermes.utils.radial_multipole_windows import calculate_radial_multipole_window_array
    from pyhermes.utils.radial_profiles import build_radial_multipole_table
    from pyhermes.utils.wavelet_grid import fourier_power_spectrum, sample_scaling_function

    J, L, box = 4, 16, 1000.0
    phi = sample_scaling_function("db2", 10)
    P = fourier_power_spectrum(phi, 0, 1, L, 1024)
    kmax = np.sqrt(3.0) * L / box
    cases = {"thick_shell": {"R": 150.0, "delta_R": 60.0}, "gaussian": {"R": 80.0},
             "gaussian_shell": {"R_shell": 150.0, "R_smooth": 40.0}, "sphere": {"R": 120.0}}
    out = {}
    for name, la in cases.items():
        for (l, m) in ((0, 0), (2, 1), (3, -2)):
            out[f"win_{name}_{l}_{m}"] = calculate_radial_multipole_window_array(L, P, la, name, l, m, box_size=box)
        for l in (1, 2, 3):
            km, tab = build_radial_multipole_table(name, la, l, kmax)
            out[f"tab_{name}_{l}"] = tab
            out[f"tabkmax_{name}_{l}"] = np.array(km)
    # the task with thick-shell bins (R from the mapping, delta_R fixed)
    rng = np.random.default_rng(23)
    pos = rng.uniform(0.0, 1000.0, (4000, 3))
    pos[:1500] = pos[:1500] * 0.3 + 350.0
    w = np.full(4000, 1.0)
    f = _projection(pos, J, weights=w)
    params = {"sfc_field": f, "random": "uniform",
              "binning_window12": {"type": "thick_shell", "len_args": {"delta_R": 50.0}, "other_args": {},
                                   "mapping": {"R": "r12"}},
              "binning_window13": {"type": "thick_shell", "len_args": {"delta_R": 50.0}, "other_args": {},
                                   "mapping": {"R": "r13"}},
              "sampling": {"mode": "paired", "r12": [150.0, 200.0], "r13": [250.0, 300.0]},
              "l_min": 0, "l_max": 2, "products": ["ddd_l", "zeta_l"], "summation_backend": "cpu"}
    d = Corr_3PCF_Multipole({"Corr_3PCF_Multipole": params}).run(save_result=False)
    _save("tabulated_J4", P=P, pos=pos, weights=w, ddd_l=d.ddd_l, delta_ddd_l=d.delta_ddd_l, zeta_l=d.zeta_l,
          rrr_l=d.rrr_l, **out)


def gen_radial_diagnostics():
    """diagnose_radial_multipole_table (utils/radial_profiles.py:559-648) for
    built-in profiles, and the multipole task's per-sample diagnostics
    (theory/corr3pcf_multipole.py:668-718) after prepare_input_fields."""
    from pyhermes.theory.corr3pcf_multipole import Corr_3PCF_Multipole
    from pyhermes.utils.radial_profiles import diagnose_radial_multipole_table

    kmax = np.sqrt(3.0) * 16 / 1000.0
    cases = [("thick_shell", {"R": 150.0, "delta_R": 60.0}, 1, {}), ("gaussian", {"R": 80.0}, 2, {}),
             ("sphere", {"R": 120.0}, 0, {}), ("gaussian_shell", {"R_shell": 150.0, "R_smooth": 40.0}, 0, {}),
             ("gaussian_shell", {"R_shell": 150.0, "R_smooth": 40.0}, 2, {"quadrature_points": 600}),
             ("shell", {"R": 100.0}, 3, {}), ("sphere", {"R": 120.0}, 1, {"table_points": 64})]
    direct = [diagnose_radial_multipole_table(k, la, l, kmax, profile_config=pc) for k, la, l, pc in cases]
    rng = np.random.default_rng(23)
    pos = rng.uniform(0.0, 1000.0, (1000, 3))
    f = _projection(pos, 4)
    task = Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field": f, "random": "uniform",
        "binning_window12": {"type": "thick_shell", "len_args": {"delta_R": 50.0}, "other_args": {},
                             "mapping": {"R": "r12"}},
        "binning_window13": {"type": "sphere", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [150.0, 200.0], "r13": [250.0, 300.0]},
        "l_min": 0, "l_max": 2, "products": ["ddd_l"], "summation_backend": "cpu"}})
    task.prepare_input_fields()
    _save("radial_diagnostics_J4", pos=pos, direct=np.array(_info_json({"d": direct})),
          task=np.array(_info_json({"d": task.radial_profile_diagnostics})))


def gen_pair_at_sample():
    """Corr_2PCF.calc_pair_product / compute_pair_product_at_sample
    (theory/corr2pcf.py:375-382, 632-645): grid-unit pair products at one
    sample, and a scalar vertex."""
    from pyhermes.theory.corr2pcf import Corr_2PCF, compute_pair_product_at_sample

    rng = np.random.default_rng(52)
    pos = rng.uniform(0.0, 1000.0, (3000, 3))
    pos[:1000] = pos[:1000] * 0.3 + 300.0
    f = _projection(pos, 4)
    bw = {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"}
    v1 = compute_pair_product_at_sample({"s": 150.0}, f, None, bw)
    task = Corr_2PCF({"Corr_2PCF": {"sfc_field": f, "binning_window": bw, "sampling": {"s": [150.0]}}})
    v2 = task.calc_pair_product({"s": 220.0}, f)
    v3 = task.calc_pair_product({"s": 220.0}, f, 2.5e-4)
    _save("pair_at_sample_J4", pos=pos, values=np.array([v1, v2, v3]))


def gen_window_file():
    from pyhermes.io.window import WindowFunc

    w = WindowFunc({"type": "gaussian", "len_args": {"R": 90.0}}, _sfc_params(4))
    kernel = w.as_array()  # the reference builds its kernel lazily; save() writes it once built
    w.save(os.path.join(HERE, "window_gaussian_J4.pkl"), overwrite=True)
    _save("window_file_J4", kernel=kernel)


SECTIONS = {"pair_at_sample": gen_pair_at_sample, "radial_diagnostics": gen_radial_diagnostics, "phi_at_pos": gen_phi_at_pos, "full_fft_windows": gen_full_fft_windows, "custom_windows": gen_custom_windows, "mc_theta": gen_mc_theta, "composite_windows": gen_composite_windows, "particle_data": gen_particle_data, "field_algebra": gen_field_algebra, "rppi": gen_rppi, "io": gen_io, "cross": gen_cross, "normalization": gen_normalization, "mc3pcf_randoms": gen_mc3pcf_randoms, "random_catalogue": gen_random_catalogue, "mc3pcf_particle": gen_mc3pcf_particle, "window_file": gen_window_file, "tabulated": gen_tabulated, "counting": gen_counting, "mc3pcf": gen_mc3pcf, "phi": gen_phi, "deposit": gen_deposit, "windows": gen_windows,
            "convolution": gen_convolution, "corr2pcf": gen_corr2pcf, "multipole": gen_multipole}


def main(argv):
    if len(argv) < 2:
        print(__doc__)
        return 2
    _setup(argv[1])
    names = argv[2:] or list(SECTIONS)
    for n in names:
        SECTIONS[n]()
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
