"""Oracle pin for the field-density interpolation (utils/wavelet_grid.py:
143-186) against the reference's own field_density_at_pos on its projected
field (tests/golden/counting_J4.npz, made by make_golden.py)."""
import os

import numpy as np

import oracle
from pyhermes_gb300.phi import sample_scaling_function

PHI = sample_scaling_function()


def test_oracle_interp_matches_reference_field_density(golden_dir):
    g = np.load(os.path.join(golden_dir, "counting_J4.npz"))
    J, L, box = 4, 16, 1000.0
    w, _ = oracle.projection_weights(g["weights"], np.ones_like(g["weights"]), "catalog")
    eps = oracle.deposit(g["pos"], w, PHI, J, box)
    nx = oracle.interp(g["query"] * (L / box), eps, PHI, J)
    np.testing.assert_allclose(nx, g["nx_grid"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(nx * (L / box) ** 3, g["nx_physical"], rtol=1e-12, atol=0)
