"""GPU multipole engine against the float64 oracle and the reference goldens.

Tolerances: a_lm fields (float32 FFT + window) within 2e-5 * max|a|;
S_m and DDD_l within 1e-4 relative to the largest |value| of the set
(the bound stated for the mixed-precision contraction); the plain
reference-form path within the same bound.
"""
import os

import numpy as np
import pytest
import torch

import oracle
from pyhermes_gb300 import multipole as mp
from pyhermes_gb300.phi import cal_gamma, sample_scaling_function
from pyhermes_gb300.window import phi_power_device, rfft_field

pytestmark = pytest.mark.gpu
PHI = sample_scaling_function()


def _field(J, seed=3, clump=True):
    rng = np.random.default_rng(seed)
    L = 1 << J
    n = 20 * L ** 3 // 8
    pos = rng.uniform(0.0, 1000.0, (n, 3))
    if clump:
        pos[: n // 3] = pos[: n // 3] * 0.3 + 350.0
    w = np.full(n, 1.0 / n)
    eps = oracle.deposit(pos, w, PHI, J, 1000.0)
    return eps - eps.mean()


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("l,m", [(0, 0), (3, 2), (4, -3), (6, 6)])
def test_multipole_fields_match_oracle(l, m):
    from scipy.fft import fftn, ifftn

    J, L = 5, 32
    eps = _field(J)
    et = torch.as_tensor(eps, dtype=torch.float32, device="cuda")
    P = phi_power_device(PHI, L, 1, 1024, "cuda")
    radii = [5.0, 9.5, 12.25]
    f = mp.multipole_fields(rfft_field(et), J, l, m, radii, P).cpu().numpy()
    Pn = oracle.fourier_power(PHI, 1, L)
    s = fftn(eps)
    for b, r in enumerate(radii):
        ref = ifftn(s * oracle.radial_multipole_window(L, Pn, r, l, m)).ravel()
        assert _rel(f[:, b], ref) < 2e-5, (l, m, b, _rel(f[:, b], ref))


def test_contract_batched_and_plain_match_oracle():
    from scipy.fft import fftn, ifftn

    J, L = 5, 32
    eps = _field(J, seed=4)
    et = torch.as_tensor(eps, dtype=torch.float32, device="cuda")
    P = phi_power_device(PHI, L, 1, 1024, "cuda")
    gam = cal_gamma(PHI, 3, 1024)
    l, m = 3, 1
    r2, r3 = [6.0, 8.5, 11.0], [7.0, 10.0]
    spec = rfft_field(et)
    f2 = mp.multipole_fields(spec, J, l, m, r2, P)
    f3 = mp.multipole_fields(spec, J, l, -m, r3, P)
    S = mp.multipole_contract(et, f2, 3, gam, J, fields3=f3, nb3=2)
    Pn = oracle.fourier_power(PHI, 1, L)
    s = fftn(eps)
    ref = np.zeros((3, 2), dtype=complex)
    for i, a in enumerate(r2):
        a2 = ifftn(s * oracle.radial_multipole_window(L, Pn, a, l, m))
        for j, b in enumerate(r3):
            a3 = ifftn(s * oracle.radial_multipole_window(L, Pn, b, l, -m))
            ref[i, j] = 4 * np.pi * oracle.contract(eps, a2, a3, gam) / L ** 3
    assert _rel(S, ref) < 1e-4, _rel(S, ref)
    # conjugate shortcut (shared field and radii) equals the explicit second batch
    f3b = mp.multipole_fields(spec, J, l, -m, r2, P)
    S1 = mp.multipole_contract(et, f2, 3, gam, J, fields3=f3b, nb3=3)
    S2 = mp.multipole_contract(et, f2, 3, gam, J, conj_sign=(-1) ** ((l + m) % 2))
    assert _rel(S2, S1) < 1e-5
    # plain reference-form path for one pair (single-radius fields)
    g2 = mp.multipole_fields(spec, J, l, m, [r2[1]], P)
    g3 = mp.multipole_fields(spec, J, l, -m, [r3[0]], P)
    assert _rel(g2.cpu().numpy(), f2[:, 1].cpu().numpy()) < 1e-5
    p = mp.multipole_contract_plain(et, g2, g3, gam, J)
    assert abs(p - ref[1, 0]) < 1e-4 * np.abs(ref).max()
    # batched contraction with single-bin ([cell]-layout) fields on one or both sides
    S11 = mp.multipole_contract(et, g2, 1, gam, J, fields3=g3, nb3=1)
    assert abs(S11[0, 0] - ref[1, 0]) < 1e-4 * np.abs(ref).max()
    S31 = mp.multipole_contract(et, f2, 3, gam, J, fields3=g3, nb3=1)
    assert _rel(S31[:, 0], ref[:, 0]) < 1e-4
    S13 = mp.multipole_contract(et, g2, 1, gam, J, fields3=f3, nb3=2)
    assert _rel(S13[0], ref[1]) < 1e-4
    g3b = mp.multipole_fields(spec, J, l, -m, [r2[1]], P)
    Sc = mp.multipole_contract(et, g2, 1, gam, J, conj_sign=(-1) ** ((l + m) % 2))
    Se = mp.multipole_contract(et, g2, 1, gam, J, fields3=g3b, nb3=1)
    assert abs(Sc[0, 0] - Se[0, 0]) < 1e-5 * abs(Se[0, 0])


def test_corr3pcf_multipole_matches_reference(golden_dir):
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "multipole_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                         "box_size": 1000.0}}).run(save_result=False)
    params = {
        "sfc_field": f, "random": "uniform",
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [150.0, 200.0], "r13": [250.0, 300.0]},
        "l_min": 0, "l_max": 2, "products": ["ddd_l", "zeta_l"]}
    for backend in ("gb300", "plain"):
        d = mp.Corr_3PCF_Multipole({"Corr_3PCF_Multipole": dict(params, summation_backend=backend)}).run(
            save_result=False)
        for k in ("ddd_l", "delta_ddd_l", "zeta_l"):
            assert _rel(getattr(d, k), g[k]) < 1e-4, (backend, k, _rel(getattr(d, k), g[k]))
        np.testing.assert_allclose(d.rrr_l, g["rrr_l"], rtol=1e-12)


def test_multipole_J6_grid_vs_oracle():
    """J=6, l <= 4, a 3x3 (r12, r13) grid: batched engine vs float64 oracle."""
    J = 6
    eps = _field(J, seed=9)
    et = torch.as_tensor(eps, dtype=torch.float32, device="cuda")
    radii = [60.0, 90.0, 120.0]
    pairs = [(a, b) for a in radii for b in radii]
    eng = mp.MultipoleEngine(et, et, et, PHI, J, 1000.0)
    got = eng.ddd(pairs, 0, 4)
    for s, (a, b) in enumerate(pairs[:3]):
        _, ref = oracle.calc_ddd_multipole(eps, eps, eps, a, b, 0, 4, PHI)
        assert _rel(got[s], ref) < 1e-4, (s, got[s], ref)


def test_mixing_solve_matches_oracle():
    """FP64 GPU mixing solve vs the float64 restatement of
    solve_multipoles_from_ratio: zeta, M and cond(M) to 1e-10 relative."""
    rng = np.random.default_rng(11)
    lmax, ns = 10, 40
    B = rng.standard_normal((ns, lmax + 1)) * 0.05
    B[:, 0] = rng.uniform(0.5, 2.0, ns)
    A = rng.standard_normal((ns, lmax + 1))
    C, M, cond = mp.mixing_solve(A, B, lmax)
    for s in range(ns):
        c_ref, m_ref, cond_ref = oracle.solve_multipoles_from_ratio(A[s], B[s], lmax)
        np.testing.assert_allclose(M[s], m_ref, rtol=1e-13, atol=1e-15)
        assert _rel(C[s], c_ref) < 1e-10
        assert abs(cond[s] - cond_ref) < 1e-10 * cond_ref


@pytest.mark.parametrize("J,l,m", [(7, 5, -2), (8, 10, 7), (9, 4, 2)])
def test_multi_bin_fields_match_single_bin(J, l, m):
    """Several bins at once (bin-major batched inverse FFT, then the
    interleave into [cell][16]) against one bin at a time ([cell] layout),
    up to J=9: the same fields within float32 rounding, 5e-6 * max|a| per
    bin, and the unused slots zero."""
    L = 1 << J
    g = torch.Generator(device="cuda").manual_seed(J)
    et = torch.randn((L, L, L), generator=g, device="cuda", dtype=torch.float32)
    spec = rfft_field(et)
    P = phi_power_device(PHI, L, 1, 1024, "cuda")
    radii = [0.0, 1.5, 3.0, 7.25, 11.0, 0.4 * L]
    f = mp.multipole_fields(spec, J, l, m, radii, P)
    assert f.shape == (L ** 3, 16)
    assert torch.count_nonzero(f[:, len(radii):]) == 0
    for b in (0, 2, 5):
        one = mp.multipole_fields(spec, J, l, m, [radii[b]], P)
        err = (f[:, b] - one).abs().max().item()
        scale = one.abs().max().item()
        assert err <= 5e-6 * max(scale, 1e-30), (J, l, m, b, err, scale)


def test_mixed_profile_bins_match_single_bins():
    """Bins on different radial profile paths in one call (thin shells, an
    analytic sphere, a tabulated thick shell at l > 0) equal one call per
    bin, and the engine's DDD with shells on r12 and spheres on r13 over a
    shared field equals its per-sample reference form."""
    J, L = 5, 32
    eps = _field(J)
    et = torch.as_tensor(eps, dtype=torch.float32, device="cuda")
    spec = rfft_field(et)
    P = phi_power_device(PHI, L, 1, 1024, "cuda")
    bins = [mp.BinSpec("shell", {"R": 150.0}), mp.BinSpec("sphere", {"R": 200.0}),
            mp.BinSpec("thick_shell", {"R": 180.0, "delta_R": 60.0}), 240.0]
    for l, m in ((0, 0), (2, 1)):
        f = mp.multipole_fields_bins(spec, J, l, m, bins, 1000.0, P)
        assert f.shape == (L ** 3, 16) and torch.count_nonzero(f[:, len(bins):]) == 0
        for b, spec_b in enumerate(bins):
            one = mp.multipole_fields_bins(spec, J, l, m, [spec_b], 1000.0, P)
            # batched and single-bin FFTs round differently: the bound of
            # test_multi_bin_fields_match_single_bin
            assert (f[:, b] - one).abs().max().item() <= 5e-6 * max(one.abs().max().item(), 1e-30), (l, m, b)
    eng = mp.MultipoleEngine(et, et, et, PHI, J, 1000.0)
    pairs = [(150.0, mp.BinSpec("sphere", {"R": 200.0})), (240.0, mp.BinSpec("sphere", {"R": 120.0}))]
    got = eng.ddd(pairs, 0, 2)
    ref = eng.ddd_plain(pairs, 0, 2)
    assert _rel(got, ref) < 1e-4


def test_corr3pcf_multipole_random_field_matches_reference(golden_dir):
    """random = a projected random catalogue: delta = D - R, rrr_l from the
    random field's own multipoles, zeta_l from the mixing solve."""
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "random_catalogue_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                         "box_size": 1000.0}}).run(save_result=False)
    r = SFCProjection({"SFCProjection": {"particle_pos": g["rpos"], "J": 4, "box_size": 1000.0}}).run(
        save_result=False)
    d = mp.Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field": f, "random": r,
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [150.0, 200.0], "r13": [250.0, 300.0]},
        "l_min": 0, "l_max": 2, "products": ["ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"]}}).run(save_result=False)
    for k in ("ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"):
        assert _rel(getattr(d, k), g["r3_" + k]) < 1e-4, (k, _rel(getattr(d, k), g["r3_" + k]))


def test_cross_fields_and_vertex_windows_match_reference(golden_dir):
    """Fields A, B, A on the three vertices, a smoothing window on vertex 2,
    grid sampling and l_min = 1 (the conjugate shortcut does not apply)."""
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "cross_J4.npz"))
    a = SFCProjection({"SFCProjection": {"particle_pos": g["pa"], "catalog_weight": g["wa"], "J": 4,
                                         "box_size": 1000.0}}).run(save_result=False)
    b = SFCProjection({"SFCProjection": {"particle_pos": g["pb"], "J": 4, "box_size": 1000.0}}).run(
        save_result=False)
    d = mp.Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field1": a, "sfc_field2": b, "sfc_field3": a, "random": "uniform",
        "window2": {"type": "gaussian", "len_args": {"R": 40.0}},
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "grid", "r12": [150.0, 200.0], "r13": [250.0]},
        "l_min": 1, "l_max": 2, "products": ["ddd_l", "delta_ddd_l"]}}).run(save_result=False)
    for k in ("ddd_l", "delta_ddd_l"):
        assert _rel(getattr(d, k), g["c3_" + k]) < 1e-4, (k, _rel(getattr(d, k), g["c3_" + k]))
