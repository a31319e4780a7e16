"""Pair products over cylindrical bins with the line of sight on z: the
column kernel (per-column z product against a table of the parallel factor,
the perpendicular factor from a table over 1/8 of the (x, y) plane) against
the generic per-mode kernel on the same bins.  70 bins of the four
cylindrical types (two groups of 64, the second padded), one to four
spectrum pairs, with and without the k = 0 mode.  The two kernels sum in
different orders in FP32 with FP64 accumulators, so the bound is 1e-5 of
each pair's largest |value| over the bins."""
import numpy as np
import pytest
import torch

from pyhermes_gb300.phi import sample_scaling_function
from pyhermes_gb300.window import WindowFunc, pair_products, rfft_field

pytestmark = pytest.mark.gpu
PHI = sample_scaling_function()


def _info(J):
    return {"J": J, "box_size": 1000.0, "phi_resolution": 1024, "wavelet_mode": "db2", "wavelet_level": 10,
            "phi_array": PHI}


def _bins(J, n, seed, los=None):
    rng = np.random.default_rng(seed)
    kinds = ("ring", "disk", "cylshell", "cylinder")
    out = []
    for b in range(n):
        p = {"type": kinds[b % 4], "len_args": {"R": float(rng.uniform(20.0, 200.0)),
                                                 "H": float(rng.uniform(10.0, 150.0))}}
        if los is not None:
            p["los_args"] = los
        out.append(WindowFunc(p, _info(J), device="cuda"))
    return out


@pytest.mark.parametrize("J,n_pairs,exclude_k0", [(6, 1, True), (6, 3, False), (7, 2, True), (7, 4, True)])
def test_column_kernel_matches_generic_kernel(J, n_pairs, exclude_k0):
    L = 1 << J
    g = torch.Generator(device="cuda").manual_seed(J * 10 + n_pairs)
    fields = [torch.exp(torch.randn((L, L, L), generator=g, device="cuda")) for _ in range(3)]
    spectra = [rfft_field(f) for f in fields]
    pairs = [(0, 0), (0, 1), (1, 2), (2, 2)][:n_pairs]
    bins = _bins(J, 70, seed=J)
    col, k0c = pair_products(spectra, pairs, bins, exclude_k0=exclude_k0)
    # one non-cylindrical bin sends every bin through the generic kernel
    extra = WindowFunc({"type": "gaussian", "len_args": {"R": 30.0}}, _info(J), device="cuda")
    gen, k0g = pair_products(spectra, pairs, bins + [extra], exclude_k0=exclude_k0)
    gen, k0g = gen[:70], k0g[:70]
    assert np.all(np.isfinite(col))
    for p in range(n_pairs):
        err = np.abs(col[:, p] - gen[:, p]).max() / np.abs(gen[:, p]).max()
        assert err < 1e-5, (p, err)
    np.testing.assert_allclose(k0c, k0g, rtol=1e-6, atol=1e-7)
    # deterministic
    col2, _ = pair_products(spectra, pairs, bins, exclude_k0=exclude_k0)
    assert np.array_equal(col, col2)
