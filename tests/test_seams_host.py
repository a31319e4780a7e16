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
}
REFERENCE_DEFAULTS = {
    "project_scaling_grid_numba": {"phi_resolution": 1024, "J": 8, "box_size": 1000.0},
    "interpolate_grid_at_pos_numba": {"dx": 0.0, "dy": 0.0, "dz": 0.0},
    "solve_multipoles_from_ratio": {"rcond_warning": 1e12},
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
