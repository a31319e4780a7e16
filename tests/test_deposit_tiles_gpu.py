"""Deposit tile shapes and the tile autotuner.

The tile only changes how the accumulation is split over CTAs: every cell
is an integer fixed-point sum, so the float32 field and the counts must be
bit-identical for every tile shape, and the autotuner (which times the
candidates on the caller's catalogue) must leave the field unchanged.
"""
import numpy as np
import pytest
import torch

from pyhermes_gb300 import autotune, kernels, synthetic
from pyhermes_gb300.phi import sample_scaling_function

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _default_tiles():
    yield
    for J in range(2, 11):
        autotune.set_deposit_tile(J, (0, 0, 0))


@pytest.mark.parametrize("J", [6, 8])
def test_every_tile_gives_the_same_field(J):
    dev = torch.device("cuda")
    pos_np, w_np = synthetic.lognormal_catalogue(300_000, box=1000.0, ng=64, device=dev)
    pos = torch.as_tensor(pos_np, device=dev)
    w = torch.as_tensor(w_np / w_np.sum(), device=dev)
    phi = torch.as_tensor(sample_scaling_function(), device=dev)
    ref, cref, _ = kernels.deposit(pos, w, J, 1000.0, phi, counts=True)
    for tile in autotune.DEPOSIT_TILES[1:]:
        autotune.set_deposit_tile(J, tile)
        got, cnt, _ = kernels.deposit(pos, w, J, 1000.0, phi, counts=True)
        assert torch.equal(got, ref), tile
        assert torch.equal(cnt, cref), tile
    autotune.set_deposit_tile(J, (0, 0, 0))
    f64, _, _ = kernels.deposit(pos, w, J, 1000.0, phi, out_dtype=torch.float64)
    autotune.set_deposit_tile(J, (16, 32, 32))
    g64, _, _ = kernels.deposit(pos, w, J, 1000.0, phi, out_dtype=torch.float64)
    assert torch.equal(f64, g64)


def test_tuner_sets_a_valid_tile_and_keeps_the_field():
    dev = torch.device("cuda")
    J = 8
    rng = np.random.default_rng(5)
    pos = torch.as_tensor(rng.uniform(0.0, 1000.0, (200_000, 3)), device=dev)
    w = torch.as_tensor(rng.lognormal(0.0, 0.3, 200_000), device=dev)
    phi = torch.as_tensor(sample_scaling_function(), device=dev)
    ref, _, _ = kernels.deposit(pos, w, J, 1000.0, phi)
    tile, ms = autotune.tune_deposit(pos, w, J, 1000.0, phi)
    assert tuple(tile) in autotune.DEPOSIT_TILES
    assert autotune.deposit_tile(J) == tuple(min(t, 1 << J) for t in tile)
    assert len(ms) >= 5 and all(v > 0 for v in ms.values())
    got, _, _ = kernels.deposit(pos, w, J, 1000.0, phi)
    assert torch.equal(got, ref)
