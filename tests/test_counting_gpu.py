"""GPU field_density_at_pos and Counting against the reference's outputs
(tests/golden/counting_J4.npz): float32 gathers, 1e-5 relative."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_field_density_and_counting_match_reference(golden_dir, tmp_path):
    from pyhermes_gb300.counting import Counting, CountingData
    from pyhermes_gb300.projection import SFCProjection
    from pyhermes_gb300.window import WindowFunc

    g = np.load(os.path.join(golden_dir, "counting_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                         "box_size": 1000.0}}).run(save_result=False)
    q = g["query"]
    assert _rel(f.field_density_at_pos(q, value_unit="physical"), g["nx_physical"]) < 1e-5
    assert _rel(f.field_density_at_pos(q, value_unit="grid"), g["nx_grid"]) < 1e-5
    win = WindowFunc({"type": "gaussian", "len_args": {"R": 80.0}}, f.sfc_info)
    assert _rel(f.field_density_at_pos(q, filter=win), g["nx_filter"]) < 1e-5
    assert _rel(f.field_density_at_pos(q, normalization="unit"), g["nx_unit"]) < 1e-5
    out = str(tmp_path / "counting.pkl")
    d = Counting({"Counting": {"sfc_field": f, "random_count": 700, "seed": 5, "fout_path": out,
                               "window": {"type": "gaussian", "len_args": {"R": 80.0}}}}).run()
    assert _rel(d.nx, g["counting_nx"]) < 1e-5
    back = CountingData(out)
    np.testing.assert_array_equal(back.nx, d.nx)
    assert back.counting_info["random_count"] == 700
