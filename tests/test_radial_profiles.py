"""Host radial-profile tables (non-shell multipole windows) against the
reference's own tables (tests/golden/tabulated_J4.npz, make_golden.py)."""
import os

import numpy as np
import pytest

from pyhermes_gb300 import radial_profiles as rp
from test_tasks_host import oracle_kernels  # noqa: F401  (fixture)

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


def _same_diagnostic(got, ref):
    assert set(got) == set(ref), (sorted(got), sorted(ref))
    for k, v in ref.items():
        if isinstance(v, float) and not isinstance(v, bool):
            assert abs(got[k] - v) <= 1e-13 + 1e-12 * abs(v), (k, got[k], v)
        else:
            assert got[k] == v, (k, got[k], v)


def test_radial_table_diagnostics_match_reference(golden_dir):
    """diagnose_radial_multipole_table (utils/radial_profiles.py:559-648):
    every field of the reference's record, a failing coarse table included."""
    import json

    from pyhermes_gb300.radial_profiles import diagnose_radial_multipole_table

    g = np.load(os.path.join(golden_dir, "radial_diagnostics_J4.npz"))
    kmax = np.sqrt(3.0) * 16 / 1000.0
    cases = [("thick_shell", {"R": 150.0, "delta_R": 60.0}, 1, {}), ("gaussian", {"R": 80.0}, 2, {}),
             ("sphere", {"R": 120.0}, 0, {}), ("gaussian_shell", {"R_shell": 150.0, "R_smooth": 40.0}, 0, {}),
             ("gaussian_shell", {"R_shell": 150.0, "R_smooth": 40.0}, 2, {"quadrature_points": 600}),
             ("shell", {"R": 100.0}, 3, {}), ("sphere", {"R": 120.0}, 1, {"table_points": 64})]
    ref = json.loads(str(g["direct"]))["d"]
    for (k, la, l, pc), r in zip(cases, ref):
        _same_diagnostic(diagnose_radial_multipole_table(k, la, l, kmax, profile_config=pc), r)


def test_task_radial_diagnostics_match_reference(golden_dir, oracle_kernels):
    """The multipole task's per-sample table diagnostics after
    prepare_input_fields (theory/corr3pcf_multipole.py:668-718), recorded in
    its info as radial_profile_diagnostics_result."""
    import json

    from pyhermes_gb300.multipole import Corr_3PCF_Multipole
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "radial_diagnostics_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "J": 4, "box_size": 1000.0}},
                      device="cpu").run(save_result=False)
    task = Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field": f, "random": "uniform",
        "binning_window12": {"type": "thick_shell", "len_args": {"delta_R": 50.0}, "other_args": {},
                             "mapping": {"R": "r12"}},
        "binning_window13": {"type": "sphere", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [150.0, 200.0], "r13": [250.0, 300.0]},
        "l_min": 0, "l_max": 2, "products": ["ddd_l"]}}, device="cpu")
    task.prepare_input_fields()
    ref = json.loads(str(g["task"]))["d"]
    assert len(task.radial_profile_diagnostics) == len(ref) == 8
    for got, r in zip(task.radial_profile_diagnostics, ref):
        _same_diagnostic(got, r)
