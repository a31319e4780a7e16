"""Degree pairs on the GPU: hermes_multipole_fields_pair_bm against the two
single-degree fields, hermes_multipole_contract_pair_bm_async against the
two single-degree contractions, and the graphed engine with and without
pairs.  The paired field differs from the two single ones only by the
rounding of their sum in the window, so the bound is FP32 rounding of the
field (2e-6 of max |a|) and 1e-5 of the largest |S| of each matrix."""
import ctypes

import numpy as np
import pytest
import torch

from pyhermes_gb300 import multipole as mp
from pyhermes_gb300 import synthetic
from pyhermes_gb300.kernels import deposit
from pyhermes_gb300.phi import cal_gamma, sample_scaling_function
from pyhermes_gb300.window import phi_power_device, rfft_field

pytestmark = pytest.mark.gpu
PHI = sample_scaling_function()
BOX = 1000.0


@pytest.fixture(scope="module")
def field():
    J = 7
    pos, w = synthetic.lognormal_catalogue(200_000, box=BOX, ng=64, device="cuda")
    pw = torch.as_tensor(w / w.sum(), device="cuda")
    eps, _, _ = deposit(torch.as_tensor(pos, device="cuda"), pw, J, BOX, torch.as_tensor(PHI, device="cuda"))
    eps = (eps - eps.double().mean().float()).contiguous()
    return J, eps


def _radii(J, nb):
    L = 1 << J
    return [r * L / BOX for r in np.linspace(20.0, 150.0, nb)]


@pytest.mark.parametrize("l,nb", [(0, 5), (2, 3), (8, 15)])
def test_pair_fields_are_the_sum_of_the_two_degrees(field, l, nb):
    J, eps = field
    L = 1 << J
    spec = rfft_field(eps)
    P = phi_power_device(PHI, L, 1, 1024, "cuda")
    radii = _radii(J, nb)
    pair = mp.multipole_fields_pair(spec, J, l, radii, P).clone()
    a = mp.multipole_fields(spec, J, l, 0, radii, P, bin_major=True).clone().view(nb, -1)
    b = mp.multipole_fields(spec, J, l + 1, 0, radii, P, bin_major=True).clone().view(nb, -1)
    for k in range(nb):
        sa, sb = a[k].abs().max().item(), b[k].abs().max().item()
        # a_{l,0} real, a_{l+1,0} imaginary: the pair carries one in each part
        assert a[k].imag.abs().max().item() <= 1e-5 * sa
        assert b[k].real.abs().max().item() <= 1e-5 * sb
        err = (pair[k] - (a[k] + b[k])).abs().max().item()
        assert err <= 2e-6 * max(sa, sb), (l, k, err, sa, sb)


@pytest.mark.parametrize("l", [0, 4])
def test_pair_contraction_matches_the_single_degrees(field, l):
    J, eps = field
    L = 1 << J
    nb = 12
    spec = rfft_field(eps)
    P = phi_power_device(PHI, L, 1, 1024, "cuda")
    radii = _radii(J, nb)
    g = (ctypes.c_double * 9)(*np.asarray(cal_gamma(PHI, 3, 1024), dtype=np.float64).ravel())
    out = torch.zeros((3, 16, 16, 2), dtype=torch.float64, device="cuda")
    f = mp.multipole_fields_pair(spec, J, l, radii, P)
    mp.multipole_contract_pair_async(eps, f, nb, g, J, out[0])
    for d in (0, 1):
        fd = mp.multipole_fields(spec, J, l + d, 0, radii, P, bin_major=True)
        mp.multipole_contract_async(eps, fd, nb, g, J, out[1 + d], conj_sign=(-1) ** ((l + d) % 2), bin_major=True)
    o = out[:, :nb, :nb].cpu().numpy()
    for d in (0, 1):
        ref = o[1 + d, ..., 0]
        assert np.abs(o[1 + d, ..., 1]).max() <= 1e-5 * np.abs(ref).max()  # m = 0 summands are real
        err = np.abs(o[0, ..., d] - ref).max() / np.abs(ref).max()
        assert err <= 1e-5, (l, d, err)


def test_graphed_engine_pairs_match_unpaired(field):
    J, eps = field
    radii = list(np.linspace(20.0, 150.0, 6))
    got = {}
    for pairs in (True, False):
        eng = mp.GraphedMultipole(J, BOX, radii, 5, PHI, "cuda", pair_degrees=pairs)
        got[pairs] = eng.summands(eps)
        if pairs:
            assert eng.pairs == [0, 2, 4]
    for k in range(got[True].shape[0]):
        ref = got[False][k]
        err = np.abs(got[True][k] - ref).max() / np.abs(ref).max()
        assert err <= 1e-5, (k, err)
