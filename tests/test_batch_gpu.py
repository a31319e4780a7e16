"""Batched uneven catalogues against the public API used one at a time.

The batch shares bin windows, runs four catalogues' pair products in one
pass and replays one CUDA graph of the multipole (l, m) loop per J with an
autotuned contraction tile.  2PCF results must match the one-at-a-time path
to 1e-9 relative (same kernels); 3PCF products to 1e-4 relative, the
bound of the mixed-precision (tensor-core) contraction: the autotuned tile
changes which cells one work item's FP32 tensor-memory accumulator sums.  A second
replay of the captured graph must reproduce the first exactly.
"""
import numpy as np
import pytest

from pyhermes_gb300 import batch

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_batch_pipeline_matches_one_at_a_time():
    cats = batch.c4_catalogues(n_cat=5, n_min=2e4, n_max=6e4, js=(5, 6), rs=(20.0, 40.0))
    radii = [100.0, 150.0, 200.0, 250.0]
    edges = np.linspace(20.0, 200.0, 6)
    ref = batch.run_one_at_a_time(cats, lmax=2, radii=radii, edges=edges)
    bp = batch.BatchPipeline(lmax=2, radii=radii, edges=edges)
    got = bp.run(cats)
    assert set(bp.tiles) == {5, 6}
    assert set(bp.deposit_tiles) == {5, 6}
    for r, g in zip(ref, got):
        assert _rel(g["xi"], r["xi"]) < 1e-9
        assert _rel(g["delta_ddd_l"], r["delta_ddd_l"]) < 1e-4
        assert _rel(g["zeta_l"], r["zeta_l"]) < 1e-4
    again = bp.run(cats)
    for g, a in zip(got, again):
        np.testing.assert_array_equal(g["delta_ddd_l"], a["delta_ddd_l"])
    nog = batch.BatchPipeline(lmax=2, radii=radii, edges=edges, use_graph=False, autotune_tiles=False).run(cats[:2])
    for r, g in zip(ref[:2], nog):
        assert _rel(g["delta_ddd_l"], r["delta_ddd_l"]) < 1e-9
