"""Particle datasets written by SFCProjection(save_particle_data=True)
(base/sfc_projection.py:195-219) and SFCField.get_particle_data from them
(io/sfc_field.py:425-482), against the reference (golden
particle_data_J4.npz, "saved" entries)."""
import os

import numpy as np

from pyhermes_gb300.projection import SFCProjection
from test_tasks_host import oracle_kernels  # noqa: F401  (fixture)


def test_saved_particle_dataset_matches_reference(golden_dir, oracle_kernels, tmp_path):
    g = np.load(os.path.join(golden_dir, "particle_data_J4.npz"))
    rng = np.random.default_rng(131)
    pos = rng.uniform(0.0, 1000.0, (400, 3))
    np.testing.assert_array_equal(pos, g["saved_pos_in"])
    s = SFCProjection({"SFCProjection": {"particle_pos": pos, "catalog_weight": rng.lognormal(0.0, 0.3, 400), "J": 4,
                                         "box_size": 1000.0, "save_particle_data": True,
                                         "particle_data_path": str(tmp_path / "p.npz")}}, device="cpu").run(
        save_result=False)
    with np.load(tmp_path / "p.npz") as z:
        assert sorted(z.files) == sorted(k.split("__")[1] for k in g.files if k.startswith("savedfile__"))
        for k in z.files:
            assert z[k].dtype == g["savedfile__" + k].dtype
            np.testing.assert_array_equal(z[k], g["savedfile__" + k])
    for k, v in s.get_particle_data().items():
        np.testing.assert_allclose(v, g["saved__" + k], rtol=1e-15, atol=0, err_msg=k)


def test_catalogue_files_are_read_by_the_caller():
    """A catalogue path without particle_pos is refused with a clear message:
    this package projects positions the caller has read."""
    import pytest

    with pytest.raises(ValueError, match="particle_pos"):
        SFCProjection({"SFCProjection": {"fin": {"path": "cat.bin", "format": "bin"}, "J": 4, "box_size": 1000.0}},
                      device="cpu").run(save_result=False)
