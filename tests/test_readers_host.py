"""Catalogue readers and SFCProjection from files against the reference
(no GPU): tests/golden/catalogues holds a small catalogue in every reader
format (bin, npz, a two-file legacy Gadget snapshot, a Gadget FoF file, a
two-file Quijote group_tab catalogue); catalogues_J4.npz holds what the
reference's read_particle_data returned for each (same keys, bit-identical
arrays) and the fields its SFCProjection built from fin (bin with weight and
value columns, FoF with masses as weights)."""
import json
import os

import numpy as np
import pytest

from pyhermes_gb300.projection import SFCProjection
from pyhermes_gb300.readers import infer_format, read_particle_data
from test_field_algebra_host import _clean, _close
from test_tasks_host import oracle_kernels  # noqa: F401  (fixture)

CASES = {
    "bin": ("cat.bin", {"format": "bin", "ncols": 5, "fields": {"weight": 3, "value": 4}}),
    "npz": ("cat.npz", {}),
    "gadget": ("snap_000", {"format": "gadget"}),
    "gadget_fof": ("fof_000", {"format": "gadget-fof"}),
    "fof_file": (os.path.join("groups_000", "group_tab_000.0"), {"redshift": 0.5}),
    "fof_dir": ("", {"format": "fof", "snapnum": 0}),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_reader_matches_reference(golden_dir, case):
    g = np.load(os.path.join(golden_dir, "catalogues_J4.npz"))
    rel, params = CASES[case]
    path = os.path.join(golden_dir, "catalogues", rel) if rel else os.path.join(golden_dir, "catalogues")
    data = read_particle_data(path, **dict(params))
    keys = {k.split("__", 1)[1] for k in g.files if k.startswith(case + "__")}
    assert set(data) == keys, (case, set(data) ^ keys)
    for k in keys:
        ref = g[f"{case}__{k}"]
        got = np.asarray(data[k])
        assert got.dtype == ref.dtype and got.shape == ref.shape, (case, k, got.dtype, ref.dtype)
        np.testing.assert_array_equal(got, ref, err_msg=f"{case}.{k}")


def test_format_inference_and_errors(golden_dir, tmp_path):
    assert infer_format("a/b/group_tab_004.12") == "fof"
    assert infer_format("x.NPZ") == "npz" and infer_format("s.gadget") == "gadget" and infer_format("x.dat") is None
    with pytest.raises(ValueError):
        read_particle_data(str(tmp_path / "x.dat"))
    with pytest.raises(ValueError):
        read_particle_data("https://example.invalid/cat.bin", "bin")
    bad = tmp_path / "odd.bin"
    np.arange(7, dtype=np.float32).tofile(bad)
    with pytest.raises(ValueError):
        read_particle_data(str(bad), "bin", ncols=3)


@pytest.mark.parametrize("name", ["proj_bin", "proj_fof"])
def test_projection_from_catalogue_file_matches_reference(golden_dir, oracle_kernels, name):
    g = np.load(os.path.join(golden_dir, "catalogues_J4.npz"))
    d = os.path.join(golden_dir, "catalogues")
    fin = {"proj_bin": {"path": os.path.join(d, "cat.bin"), "format": "bin",
                        "reader_params": {"ncols": 5, "fields": {"weight": 3, "value": 4}},
                        "catalog_weight_key": "weight", "field_value_key": "value"},
           "proj_fof": {"path": os.path.join(d, "groups_000", "group_tab_000.0"), "format": "fof",
                        "reader_params": {"fields": {"mass": "mass"}}, "catalog_weight_key": "mass"}}[name]
    f = SFCProjection({"SFCProjection": {"fin": fin, "J": 4, "box_size": 1000.0, "weight_normalization": "catalog"}},
                      device="cpu").run(save_result=False)
    ref = g[name + "__epsilon"]
    assert np.abs(np.asarray(f.epsilon) - ref).max() <= 2e-6 * np.abs(ref).max()
    _close(_clean({k: v for k, v in f.sfc_info.items() if k != "fin"}), json.loads(str(g[name + "__info"])), name)
    _close(_clean({k: v for k, v in f.sfc_info["fin"].items() if k != "path"}), json.loads(str(g[name + "__fin"])),
           name + ".fin")
