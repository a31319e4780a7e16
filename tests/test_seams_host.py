"""The kernel-seam module (no GPU): every seam the reference's task classes
call by name exists with the reference's parameter names and defaults, and
the per-sample binning-window conversion follows the reference's radial
profiles."""
import inspect

import pytest

from pyhermes_gb300 import seams
from pyhermes_gb300.multipole import BinSpec

# parameter lists of the reference seams (file:line in the reference project)
REFERENCE_SIGNATURES = {
    # pyhermes/utils/wavelet_grid.py:59-65
    "project_scaling_grid_numba": ["positions", "weights", "phi_array", "phi_resolution", "J", "box_size"],
    # pyhermes/utils/wavelet_grid.py:144-154
    "interpolate_grid_at_pos_numba": ["output_values", "scaled_positions", "grid_values", "phi_array", "grid_size",
                                      "phi_resolution", "phi_support", "dx", "dy", "dz"],
    # pyhermes/utils/convolution.py:284
    "specialized_convolution_3d": ["s", "w", "threads"],
    # pyhermes/theory/corr2pcf.py:366
    "pair_product_with_window": ["field1", "field2", "binning_window_obj", "threads"],
    # pyhermes/utils/corr3pcf_multipoles.py:460-472
    "calc_DDD_multipole": ["deltaD1", "deltaD2", "deltaD3", "binning_window12", "binning_window13", "l_min", "l_max",
                           "summation_backend", "gpu_device_id", "gpu_threads_per_block", "cache_multipole_fields",
                           "cache_dir", "cache_namespace", "threads", "progress_callback", "m_progress_callback"],
    # pyhermes/utils/special_functions.py:392
    "solve_multipoles_from_ratio": ["A", "B", "lmax", "rcond_warning"],
    # pyhermes/utils/corr3pcf_multipoles.py:393
    "compute_multipole_m_summand": ["field_r1_m", "field_r2_m", "sum_context"],
    # pyhermes/theory/corr3pcf.py:68-78
    "estimate_triplet_product_with_sampled_centers": ["r12_scaled", "r13_scaled", "mu", "center_scaled", "n_rot",
                                                      "sfc_meta", "sfc_field2", "sfc_field3", "center",
                                                      "center_weight", "center_weight_sum", "seed_base_rot",
                                                      "mu_index", "eps1", "rho1"],
}
REFERENCE_DEFAULTS = {
    "project_scaling_grid_numba": {"phi_resolution": 1024, "J": 8, "box_size": 1000.0},
    "interpolate_grid_at_pos_numba": {"dx": 0.0, "dy": 0.0, "dz": 0.0},
    "solve_multipoles_from_ratio": {"rcond_warning": 1e12},
    "estimate_triplet_product_with_sampled_centers": {"center": "box_random", "center_weight": None,
                                                      "center_weight_sum": None, "seed_base_rot": -1,
                                                      "mu_index": -1, "eps1": None, "rho1": None},
}


@pytest.mark.parametrize("name", sorted(REFERENCE_SIGNATURES))
def test_seam_signature(name):
    fn = getattr(seams, name)
    params = inspect.signature(fn).parameters
    assert list(params) == REFERENCE_SIGNATURES[name]
    for k, v in REFERENCE_DEFAULTS.get(name, {}).items():
        assert params[k].default == v, (name, k)
    assert name in seams.__all__


def test_radial_bin_conversion():
    assert seams._radial_bin({"type": "shell", "len_args": {"R": 42.0}}) == 42.0
    b = seams._radial_bin({"type": "thick_shell", "len_args": {"R": 40.0, "delta_R": 5.0}, "other_args": {}})
    assert isinstance(b, BinSpec) and b.type == "thick_shell" and b.len_args == {"R": 40.0, "delta_R": 5.0}
    with pytest.raises(ValueError):
        seams._radial_bin({"type": "cubic", "len_args": {"R": 1.0}})
    with pytest.raises(ValueError):
        seams._radial_bin({"type": "shell", "len_args": {"R": None}})


def test_seam_argument_checks_on_host():
    import numpy as np

    with pytest.raises(ValueError):
        seams._level(48)
    with pytest.raises(ValueError):  # raised before any device work, as in the reference
        seams.calc_DDD_multipole(None, None, None, {}, {}, 3, 2)
    with pytest.raises(ValueError):
        seams.solve_multipoles_from_ratio(np.ones(2), np.ones(2), 3)
    with pytest.raises(ValueError):
        seams.interpolate_grid_at_pos_numba(np.zeros(1), np.zeros((1, 3)), np.zeros((4, 4, 4)), np.ones(8), 4, 2, 2)


def test_mc_seam_matches_oracle(monkeypatch):
    """estimate_triplet_product_with_sampled_centers with the triplet kernel
    replaced by the oracle's interpolation (CPU tensors): box-random centres
    against oracle.mc_box_random, particle centres against the same sum
    written out with the reference's per-rotation seeds."""
    from types import SimpleNamespace

    import numpy as np
    import torch

    import oracle
    from pyhermes_gb300 import mc3pcf
    from pyhermes_gb300.phi import sample_scaling_function
    from test_tasks_host import _cpu_triplet_sum

    monkeypatch.setattr(mc3pcf, "triplet_sum", _cpu_triplet_sum)
    monkeypatch.setattr(seams, "_device", lambda: torch.device("cpu"))
    phi = sample_scaling_function()
    J, L = 5, 32
    rng = np.random.default_rng(5)
    e1, e2, e3 = (oracle.deposit(rng.uniform(0, 1000, (8000, 3)), np.full(8000, 1 / 8000), phi, J, 1000.0)
                  for _ in range(3))
    centres = rng.uniform(0.0, L, (300, 3))
    meta = SimpleNamespace(L=L, phi_array=phi, phi_resolution=1024, phi_support=3)
    got = seams.estimate_triplet_product_with_sampled_centers(4.8, 8.0, 0.3, centres, 4, meta, e2, e3,
                                                              seed_base_rot=5, mu_index=2, eps1=e1)
    ref = oracle.mc_box_random(e1, e2, e3, J, centres, 4.8, 8.0, 0.3, 4, 5, 2, phi)
    assert abs(got - ref) <= 1e-5 * abs(ref)
    w = rng.uniform(0.5, 1.5, 300)
    got = seams.estimate_triplet_product_with_sampled_centers(4.8, 8.0, -0.6, centres, 3, meta, e2, e3,
                                                              center="particle", center_weight=w,
                                                              seed_base_rot=9, mu_index=0, rho1=2.0)
    total = 0.0
    for irot in range(3):
        np.random.seed(9 + irot)
        a, b, c = np.random.rand(3)
        o = oracle.generate_triangle_offsets(4.8, 8.0, -0.6, 2 * np.pi * a, 2 * b - 1, 2 * np.pi * c)
        total += float(np.sum(w * oracle.interp(centres, e2, phi, J, offset=o[0:3])
                              * oracle.interp(centres, e3, phi, J, offset=o[3:6])))
    ref = 2.0 * total / (3 * w.sum())
    assert abs(got - ref) <= 1e-5 * abs(ref)
    with pytest.raises(ValueError):
        seams.estimate_triplet_product_with_sampled_centers(4.8, 8.0, 0.3, centres, 1, meta, e2, e3)
