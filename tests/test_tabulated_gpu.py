"""Non-shell radial multipole windows on the GPU (analytic l = 0 transfers and
host U_l(k) tables with the device local cubic) against the reference's own
window arrays and its Corr_3PCF_Multipole with thick-shell bins
(tests/golden/tabulated_J4.npz).  Fields within 2e-5 of max|a|; task
products within 1e-4 relative."""
import os

import numpy as np
import pytest
import torch

import oracle
from pyhermes_gb300 import multipole as mp
from pyhermes_gb300.phi import sample_scaling_function
from pyhermes_gb300.window import phi_power_device, rfft_field

pytestmark = pytest.mark.gpu
PHI = sample_scaling_function()
CASES = {"thick_shell": {"R": 150.0, "delta_R": 60.0}, "gaussian": {"R": 80.0},
         "gaussian_shell": {"R_shell": 150.0, "R_smooth": 40.0}, "sphere": {"R": 120.0}}


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("name", sorted(CASES))
def test_profile_fields_match_reference_windows(golden_dir, name):
    from scipy.fft import fftn, ifftn

    g = np.load(os.path.join(golden_dir, "tabulated_J4.npz"))
    J, L = 4, 16
    rng = np.random.default_rng(3)
    pos = rng.uniform(0.0, 1000.0, (3000, 3))
    eps = oracle.deposit(pos, np.full(3000, 1.0 / 3000), PHI, J, 1000.0)
    eps = eps - eps.mean()
    et = torch.as_tensor(eps, dtype=torch.float32, device="cuda")
    P = phi_power_device(PHI, L, 1, 1024, "cuda")
    spec = rfft_field(et)
    s = fftn(eps)
    for (l, m) in ((0, 0), (2, 1), (3, -2)):
        f = mp.multipole_fields_bins(spec, J, l, m, [mp.BinSpec(name, CASES[name])], 1000.0, P).cpu().numpy()
        ref = ifftn(s * g[f"win_{name}_{l}_{m}"]).ravel()
        assert _rel(f, ref) < 2e-5, (name, l, m, _rel(f, ref))
    # several bins in one call, bin-interleaved
    bins = [mp.BinSpec(name, CASES[name]), mp.BinSpec(name, CASES[name])]
    f2 = mp.multipole_fields_bins(spec, J, 2, 1, bins, 1000.0, P).cpu().numpy()
    ref = ifftn(s * g[f"win_{name}_2_1"]).ravel()
    assert _rel(f2[:, 0], ref) < 2e-5 and _rel(f2[:, 1], ref) < 2e-5


def test_corr3pcf_multipole_thick_shell_matches_reference(golden_dir):
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "tabulated_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                         "box_size": 1000.0}}).run(save_result=False)
    params = {
        "sfc_field": f, "random": "uniform",
        "binning_window12": {"type": "thick_shell", "len_args": {"delta_R": 50.0}, "other_args": {},
                             "mapping": {"R": "r12"}},
        "binning_window13": {"type": "thick_shell", "len_args": {"delta_R": 50.0}, "other_args": {},
                             "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [150.0, 200.0], "r13": [250.0, 300.0]},
        "l_min": 0, "l_max": 2, "products": ["ddd_l", "zeta_l"]}
    for backend in ("gb300", "plain"):
        d = mp.Corr_3PCF_Multipole({"Corr_3PCF_Multipole": dict(params, summation_backend=backend)}).run(
            save_result=False)
        for k in ("ddd_l", "delta_ddd_l", "zeta_l"):
            assert _rel(getattr(d, k), g[k]) < 1e-4, (backend, k, _rel(getattr(d, k), g[k]))
