"""The oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the unmodified reference)."""
import os

import numpy as np
import pytest

import oracle
from pyhermes_gb300 import phi as phimod


def _load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name + ".npz"))


def test_phi_cascade_matches_reference(golden_dir):
    g = _load(golden_dir, "phi_db2")
    phi = phimod.sample_scaling_function("db2", 10)
    assert phi.shape == (3072,)
    np.testing.assert_array_equal(phi, g["phi"])
    # scaling-function invariants: unit integral and partition of unity
    assert abs(phi.sum() / 1024 - 1.0) < 1e-12
    pou = phi.reshape(3, 1024).sum(axis=0)
    assert np.max(np.abs(pou - 1.0)) < 1e-9


def test_fourier_power_and_gamma_match_reference(golden_dir):
    g = _load(golden_dir, "phi_db2")
    phi = g["phi"]
    np.testing.assert_array_equal(phimod.fourier_power_spectrum(phi, 1, 16, 1024), g["power_L16"])
    np.testing.assert_array_equal(phimod.fourier_power_spectrum(phi, 2, 64, 1024), g["power_L32_bw2"])
    gam = phimod.cal_gamma(phi, 3, 1024)
    np.testing.assert_array_equal(gam, g["gamma"])
    assert abs(gam.sum() - 1.0) < 1e-12


@pytest.mark.parametrize("name", ["uniform_J4", "weighted_J5", "single_raw_J4"])
def test_oracle_deposit_bit_exact(golden_dir, name):
    d = _load(golden_dir, "deposit_" + name)
    phi = _load(golden_dir, "phi_db2")["phi"]
    pw, fi = oracle.projection_weights(d["catalog_weight"], d["field_value"], str(d["mode"]))
    eps = oracle.deposit(d["pos"], pw, phi, int(d["J"]), float(d["box"]))
    np.testing.assert_array_equal(eps, d["epsilon"])
    assert fi == float(d["field_integral"])
    # deposit conserves the field integral (partition of unity)
    assert abs(eps.sum() - fi) < 1e-12 * max(1.0, abs(fi))


def test_oracle_cell_counts_total(golden_dir):
    d = _load(golden_dir, "deposit_weighted_J5")
    c = oracle.cell_counts(d["pos"], int(d["J"]), float(d["box"]))
    assert int(c.sum()) == d["pos"].shape[0]
