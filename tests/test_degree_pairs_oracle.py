"""The identities the degree pairs rest on, in float64 with the oracle on a
16^3 grid: a_{l,0} = ifftn(eps_hat K_{l,0}) is real for even l and
imaginary for odd l; the field of the summed window K_{l,0} + K_{l+1,0}
(l even) carries a_{l,0} in its real part and a_{l+1,0}/i in its imaginary
part; and with a3 = conj(c) the product of the real parts is S_{l,0} while
the product of the imaginary parts, sum v2 G(-v3), is S_{l+1,0} -- the two
blocks the packed contraction epilogue returns."""
import numpy as np
import pytest
from scipy.fft import fftn, ifftn

import oracle

L = 16


@pytest.fixture(scope="module")
def setup(golden_dir):
    import os

    phi = np.load(os.path.join(golden_dir, "phi_db2.npz"))["phi"]
    rng = np.random.default_rng(11)
    eps = rng.standard_normal((L, L, L))
    return eps, fftn(eps), oracle.fourier_power(phi, 1, L), oracle.cal_gamma(phi)


@pytest.mark.parametrize("l", [0, 2, 4])
def test_pair_field_carries_both_degrees(setup, l):
    _, s, P, _ = setup
    r = 3.5
    ka = oracle.radial_multipole_window(L, P, r, l, 0)
    kb = oracle.radial_multipole_window(L, P, r, l + 1, 0)
    a, b, c = ifftn(s * ka), ifftn(s * kb), ifftn(s * (ka + kb))
    sa, sb = np.abs(a).max(), np.abs(b).max()
    assert np.abs(a.imag).max() <= 1e-12 * sa  # even degree: real
    assert np.abs(b.real).max() <= 1e-12 * sb  # odd degree: imaginary
    assert np.abs(c.real - a.real).max() <= 1e-12 * max(sa, sb)
    assert np.abs(c.imag - b.imag).max() <= 1e-12 * max(sa, sb)


@pytest.mark.parametrize("l", [0, 2])
def test_packed_blocks_are_the_two_summands(setup, l):
    eps, s, P, gamma = setup
    r12, r13 = 2.5, 4.0

    def fields(d, r):
        return ifftn(s * oracle.radial_multipole_window(L, P, r, d, 0))

    def pair(r):
        return ifftn(s * (oracle.radial_multipole_window(L, P, r, l, 0) +
                          oracle.radial_multipole_window(L, P, r, l + 1, 0)))

    # the m = 0 summands as calc_DDD_multipole forms them (a3 = a_{l,-0} = a_{l,0})
    s_l = oracle.contract(eps, fields(l, r12), fields(l, r13), gamma)
    s_l1 = oracle.contract(eps, fields(l + 1, r12), fields(l + 1, r13), gamma)
    c12, c13 = pair(r12), pair(r13)
    # packed epilogue, a3 = conj(c13): real-part block and imaginary-part block
    re_block = oracle.contract(eps, c12.real.astype(complex), c13.real.astype(complex), gamma)
    im_block = oracle.contract(eps, c12.imag.astype(complex), -c13.imag.astype(complex), gamma)
    scale = max(abs(s_l), abs(s_l1))
    assert abs(re_block - s_l) <= 1e-10 * scale
    assert abs(im_block - s_l1) <= 1e-10 * scale
    assert abs(s_l.imag) <= 1e-10 * scale and abs(s_l1.imag) <= 1e-10 * scale  # m = 0 summands are real
