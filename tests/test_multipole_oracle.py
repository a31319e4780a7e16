"""Oracle multipole pieces against the reference's outputs (golden
fixtures): spherical Bessel, Y_lm, radial multipole windows, DDD_l and
zeta_l at J=4, l <= 2."""
import os

import numpy as np
import pytest

import oracle


@pytest.fixture(scope="module")
def g(golden_dir):
    return np.load(os.path.join(golden_dir, "multipole_J4.npz"))


@pytest.fixture(scope="module")
def phi(golden_dir):
    return np.load(os.path.join(golden_dir, "phi_db2.npz"))["phi"]


def test_special_functions(g):
    lb = oracle._setup_multipole_lib()
    jn = np.array([[lb.oracle_spherical_jn(l, x) for x in g["jn_x"]] for l in range(11)])
    np.testing.assert_allclose(jn, g["jn"], rtol=1e-13, atol=1e-300)
    import ctypes

    for l in range(5):
        for mi, m in enumerate(range(-l, l + 1)):
            for ki, k in enumerate(g["ylm_k"]):
                re, im = ctypes.c_double(), ctypes.c_double()
                lb.oracle_sph_harm(l, m, *k, ctypes.byref(re), ctypes.byref(im))
                assert abs(complex(re.value, im.value) - g["ylm"][l, mi, ki]) < 1e-14


@pytest.mark.parametrize("key", ["window_l0_m0", "window_l2_m1", "window_l3_m-2", "window_l4_m4"])
def test_radial_multipole_window(g, phi, key):
    l = int(key.split("_l")[1].split("_")[0])
    m = int(key.split("_m")[1])
    P = oracle.fourier_power(phi, 1, 16)
    w = oracle.radial_multipole_window(16, P, 180.0 * 16 / 1000, l, m)
    np.testing.assert_allclose(w, g[key], rtol=0, atol=1e-14 * np.abs(g[key]).max())


def test_ddd_and_zeta_match_reference(g, phi):
    eps = g["epsilon"]
    rho = 1.0 / 16 ** 3
    sf9 = (16 / 1000.0) ** 9
    for s, (r12, r13) in enumerate([(150.0, 250.0), (200.0, 300.0)]):
        _, d = oracle.calc_ddd_multipole(eps, eps, eps, r12, r13, 0, 2, phi)
        np.testing.assert_allclose(d * sf9, g["ddd_l"][s], rtol=1e-12)
        _, dd = oracle.calc_ddd_multipole(eps - rho, eps - rho, eps - rho, r12, r13, 0, 2, phi)
        np.testing.assert_allclose(dd * sf9, g["delta_ddd_l"][s], rtol=1e-11, atol=1e-12 * np.abs(g["delta_ddd_l"][s]).max())
        z, _, cond = oracle.solve_multipoles_from_ratio(dd * sf9, g["rrr_l"][s], 2)
        np.testing.assert_allclose(z, g["zeta_l"][s], rtol=1e-11, atol=1e-12 * np.abs(g["zeta_l"][s]).max())
        assert abs(cond - g["zeta_condition"][s]) < 1e-9
