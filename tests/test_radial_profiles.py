"""Host radial-profile tables (non-shell multipole windows) against the
reference's own tables (tests/golden/tabulated_J4.npz, make_golden.py)."""
import os

import numpy as np
import pytest

from pyhermes_gb300 import radial_profiles as rp

CASES = {"thick_shell": {"R": 150.0, "delta_R": 60.0}, "gaussian": {"R": 80.0},
         "gaussian_shell": {"R_shell": 150.0, "R_smooth": 40.0}, "sphere": {"R": 120.0}}


@pytest.mark.parametrize("name", sorted(CASES))
def test_tables_match_reference(golden_dir, name):
    g = np.load(os.path.join(golden_dir, "tabulated_J4.npz"))
    kmax = np.sqrt(3.0) * 16 / 1000.0
    for l in (1, 2, 3):
        km, tab = rp.build_radial_multipole_table(name, CASES[name], l, kmax)
        ref = g[f"tab_{name}_{l}"]
        assert km == float(g[f"tabkmax_{name}_{l}"])
        assert tab.shape == ref.shape
        np.testing.assert_allclose(tab, ref, rtol=1e-12, atol=1e-15 * np.abs(ref).max())


def test_profile_modes_and_custom_profiles():
    assert rp.profile_mode("shell", {"R": 10.0}, 3) == "shell"
    assert rp.profile_mode("gaussian_shell", {"R_shell": 10.0, "R_smooth": 0.0}, 2) == "shell"
    assert rp.profile_mode("thick_shell", {"R": 10.0, "delta_R": 2.0}, 0) == "analytic"
    assert rp.profile_mode("thick_shell", {"R": 10.0, "delta_R": 2.0}, 1) == "table"
    # a user real profile equal to the built-in thick shell gives the same table
    lo, hi = 120.0, 180.0

    def shell(r, **kw):
        return np.where((r >= lo) & (r <= hi), 1.0, 0.0)

    prof = rp.real_space_profile(shell, hi, r_min=lo)
    kmax = np.sqrt(3.0) * 16 / 1000.0
    _, t_custom = rp.build_radial_multipole_table("custom_real", {}, 2, kmax, {"profile": prof})
    _, t_builtin = rp.build_radial_multipole_table("thick_shell", {"R": 150.0, "delta_R": 60.0}, 2, kmax)
    np.testing.assert_allclose(t_custom, t_builtin, rtol=1e-10, atol=1e-14)
