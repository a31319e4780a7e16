"""The kernel seams (pyhermes_gb300.seams) on the GPU against the float64
oracle, called with this package's objects and with stand-ins for the
reference's (NumPy ``epsilon`` fields, windows with ``window_params`` and
``as_array``).  Bounds are those of the underlying paths: deposit
|d| <= 2e-6 max|eps|; interpolation 2e-6 of max|n|; convolution 1e-5 of
max|ref|; pair products 1e-5 relative; DDD_l 1e-4 of max|DDD_l|; mixing
solve 1e-10."""
import numpy as np
import pytest

import oracle
from pyhermes_gb300 import seams
from pyhermes_gb300.phi import sample_scaling_function
from pyhermes_gb300.sfc_field import SFCField
from pyhermes_gb300.window import WindowFunc

pytestmark = pytest.mark.gpu
PHI = sample_scaling_function()


def _sfc(J):
    return {"J": J, "box_size": 1000.0, "phi_resolution": 1024, "wavelet_mode": "db2", "wavelet_level": 10}


def _info(eps, J):
    return {**_sfc(J), "L": 1 << J, "V": (1 << J) ** 3, "scale_factor": (1 << J) / 1000.0,
            "field_kind": "derived_field", "field_integral": float(eps.sum()), "phi_array": PHI, "phi_support": 3}


def _field_from(eps, J):
    import torch

    f = SFCField()
    f.sfc_info = _info(eps, J)
    f.format_sfc_params()
    f.epsilon = torch.as_tensor(eps, dtype=torch.float32, device="cuda")
    return f


class _RefLikeField:
    """What the seams see of the reference's SFCField: a float64 NumPy
    epsilon and the sfc_info keys as attributes."""

    def __init__(self, eps, J):
        self.epsilon = np.asarray(eps, dtype=np.float64)
        self.sfc_info = _info(eps, J)
        for k, v in self.sfc_info.items():
            setattr(self, k, v)

    def field_mean_density(self, value_unit="grid"):
        return None


class _RefLikeWindow:
    """What the seams see of the reference's WindowFunc."""

    def __init__(self, params, kernel):
        self.window_params = dict(params)
        self.phi_array = PHI
        self.bandwidth = 1
        self._k = kernel

    def as_array(self):
        return self._k


def _uniform_field(seed, J, n=20000):
    rng = np.random.default_rng(seed)
    return oracle.deposit(rng.uniform(0.0, 1000.0, (n, 3)), np.full(n, 1.0 / n), PHI, J, 1000.0)


def test_project_scaling_grid_matches_oracle():
    rng = np.random.default_rng(21)
    pos = rng.uniform(0.0, 1000.0, (20000, 3))
    w = rng.uniform(0.5, 1.5, 20000)
    got = seams.project_scaling_grid_numba(pos, w, PHI, 1024, 5, 1000.0)
    ref = oracle.deposit(pos, w, PHI, 5, 1000.0)
    assert got.dtype == np.float64 and got.shape == (32, 32, 32)
    assert np.abs(got - ref).max() <= 2e-6 * np.abs(ref).max()


def test_interpolate_grid_matches_oracle():
    J = 6
    eps = _uniform_field(22, J, 30000)
    pts = np.random.default_rng(23).uniform(0.0, 64.0, (5000, 3))
    out = np.zeros(5000)
    assert seams.interpolate_grid_at_pos_numba(out, pts, eps, PHI, 64, 1024, 3, 1.25, -3.5, 70.0) is None
    ref = oracle.interp(pts, eps, PHI, J, offset=(1.25, -3.5, 70.0))
    assert np.abs(out - ref).max() <= 2e-6 * np.abs(ref).max()


def test_specialized_convolution_matches_oracle():
    from scipy.fft import rfftn

    J, L = 5, 32
    rng = np.random.default_rng(24)
    s = rng.standard_normal((L, L, L))
    K = oracle.window_kernel("gaussian", {"R": 20.0}, L, oracle.fourier_power(PHI, 1, L))
    ref = oracle.convolve(s, K)
    got = seams.specialized_convolution_3d(s, K, 1)
    assert got.dtype == np.float64 and got.shape == s.shape
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    K2 = rfftn(rng.standard_normal((L, L, L))) / L ** 3  # a complex kernel of a real filter
    ref2 = oracle.convolve(s, K2)
    got2 = seams.specialized_convolution_3d(s, K2, 1)
    assert np.abs(got2 - ref2).max() <= 1e-5 * np.abs(ref2).max()


def test_pair_product_with_window_matches_oracle():
    J, L = 5, 32
    e1, e2 = _uniform_field(25, J), _uniform_field(26, J)
    params = {"type": "thick_shell", "len_args": {"R": 60.0, "delta_R": 20.0}}
    K = oracle.window_kernel("thick_shell", {"R": 60.0, "delta_R": 20.0}, L, oracle.fourier_power(PHI, 1, L))
    f1, f2 = _field_from(e1, J), _field_from(e2, J)
    w = WindowFunc(dict(params), f1.sfc_info)
    for a, b, ea, eb in [(f1, f2, e1, e2), (f1, None, e1, e1)]:
        ref = oracle.pair_product(ea, eb, K)
        got = seams.pair_product_with_window(a, b, w, 1)
        assert abs(got - ref) <= 1e-5 * abs(ref), (got, ref)
    ref = oracle.pair_product(e1, e2, K)
    got = seams.pair_product_with_window(_RefLikeField(e1, J), _RefLikeField(e2, J), _RefLikeWindow(params, K), 1)
    assert abs(got - ref) <= 1e-5 * abs(ref), (got, ref)
    assert seams.pair_product_with_window(2.0, 3.0, w, 1) == 6.0


def test_calc_ddd_multipole_matches_oracle():
    J, L = 5, 32
    rng = np.random.default_rng(27)
    n = 20 * L ** 3 // 8
    pos = rng.uniform(0.0, 1000.0, (n, 3))
    pos[: n // 3] = pos[: n // 3] * 0.3 + 350.0
    eps = oracle.deposit(pos, np.full(n, 1.0 / n), PHI, J, 1000.0)
    eps = eps - eps.mean()
    bw12 = {"type": "shell", "len_args": {"R": 150.0}}
    bw13 = {"type": "shell", "len_args": {"R": 250.0}}
    _, ref = oracle.calc_ddd_multipole(eps, eps, eps, 150.0, 250.0, 0, 3, PHI)
    f = _field_from(eps, J)
    calls = []
    lv, ddd, timing = seams.calc_DDD_multipole(f, f, f, bw12, bw13, 0, 3,
                                               progress_callback=lambda **kw: calls.append(kw))
    assert lv.dtype == np.int32 and list(lv) == [0, 1, 2, 3]
    assert np.abs(ddd - ref).max() <= 1e-4 * np.abs(ref).max(), (ddd, ref)
    assert [c["l"] for c in calls] == [0, 1, 2, 3] and calls[-1]["completed_m_tasks"] == 10
    assert {"conv_elapsed_sec", "sum_elapsed_sec"} <= set(timing)
    rf = _RefLikeField(eps, J)
    _, ddd2, _ = seams.calc_DDD_multipole(rf, rf, rf, bw12, bw13, 0, 3, summation_backend="plain")
    assert np.abs(ddd2 - ref).max() <= 1e-4 * np.abs(ref).max(), (ddd2, ref)


def test_solve_multipoles_from_ratio_matches_oracle(capsys):
    rng = np.random.default_rng(28)
    lmax = 6
    B = rng.standard_normal(lmax + 3) * 0.05
    B[0] = 1.3
    A = rng.standard_normal(lmax + 3)
    C, M, cond = seams.solve_multipoles_from_ratio(A, B, lmax)
    c_ref, m_ref, cond_ref = oracle.solve_multipoles_from_ratio(A, B, lmax)
    np.testing.assert_allclose(M, m_ref, rtol=1e-13, atol=1e-15)
    assert np.abs(C - c_ref).max() <= 1e-10 * np.abs(c_ref).max()
    assert abs(cond - cond_ref) <= 1e-10 * cond_ref
    seams.solve_multipoles_from_ratio(A, B, lmax, rcond_warning=0.5)
    assert "ill-conditioned" in capsys.readouterr().out


def test_mc_seam_matches_oracle():
    from types import SimpleNamespace

    J, L = 5, 32
    e1, e2, e3 = (_uniform_field(s, J, 8000) for s in (31, 32, 33))
    centres = np.random.default_rng(34).uniform(0.0, L, (300, 3))
    meta = SimpleNamespace(L=L, phi_array=PHI, phi_resolution=1024, phi_support=3)
    got = seams.estimate_triplet_product_with_sampled_centers(4.8, 8.0, 0.3, centres, 4, meta, e2, e3,
                                                              seed_base_rot=5, mu_index=2, eps1=e1)
    ref = oracle.mc_box_random(e1, e2, e3, J, centres, 4.8, 8.0, 0.3, 4, 5, 2, PHI)
    assert abs(got - ref) <= 1e-5 * abs(ref), (got, ref)


def test_m_summand_seam_matches_oracle():
    """compute_multipole_m_summand with the reference's cpu-style context
    against the oracle's 729-term contraction of the same fields."""
    from scipy.fft import fftn, ifftn

    J, L = 5, 32
    eps = _uniform_field(35, J)
    eps = eps - eps.mean()
    P = oracle.fourier_power(PHI, 1, L)
    s = fftn(eps)
    a2 = ifftn(s * oracle.radial_multipole_window(L, P, 5.0, 3, 1))
    a3 = ifftn(s * oracle.radial_multipole_window(L, P, 7.5, 3, -1))
    gamma = oracle.cal_gamma(PHI)
    ctx = {"backend": "cpu", "gamma": gamma, "data": eps, "n_result": eps.size, "L": L, "phi_support": 3}
    val, timing = seams.compute_multipole_m_summand(a2, a3, ctx)
    ref = 4 * np.pi * oracle.contract(eps, a2, a3, gamma) / L ** 3
    assert abs(val - ref) <= 1e-4 * abs(ref), (val, ref)
    assert set(timing) == {"h2d_elapsed_sec", "kernel_elapsed_sec", "reduce_elapsed_sec", "d2h_elapsed_sec"}
