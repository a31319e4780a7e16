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


def _bin_fin(golden_dir):
    return {"path": os.path.join(golden_dir, "catalogues", "cat.bin"), "format": "bin",
            "reader_params": {"ncols": 5, "fields": {"weight": 3, "value": 4}},
            "catalog_weight_key": "weight", "field_value_key": "value"}


def test_get_particle_data_matches_reference(golden_dir, oracle_kernels, tmp_path):
    """From the fin catalogue (field normalisation) and from a saved
    particle dataset (save_particle_data)."""
    g = np.load(os.path.join(golden_dir, "particle_data_J4.npz"))
    f = SFCProjection({"SFCProjection": {"fin": _bin_fin(golden_dir), "J": 4, "box_size": 1000.0,
                                         "weight_normalization": "field"}}, device="cpu").run(save_result=False)
    for k, v in f.get_particle_data().items():
        np.testing.assert_allclose(v, g["fin__" + k], rtol=1e-15, atol=0, err_msg=k)
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


def test_corr3pcf_particle_centres_from_field_catalogue(golden_dir, oracle_kernels, monkeypatch):
    """center='particle' without particle_pos1: the centres and projection
    weights come from sfc_field1's catalogue (re-read through fin)."""
    from pyhermes_gb300 import mc3pcf
    from test_tasks_host import _cpu_triplet_sum

    monkeypatch.setattr(mc3pcf, "triplet_sum", _cpu_triplet_sum)
    g = np.load(os.path.join(golden_dir, "particle_data_J4.npz"))
    f = SFCProjection({"SFCProjection": {"fin": _bin_fin(golden_dir), "J": 4, "box_size": 1000.0,
                                         "weight_normalization": "field"}}, device="cpu").run(save_result=False)
    d = mc3pcf.Corr_3PCF({"Corr_3PCF": {
        "sfc_field": f, "random": "uniform", "r12": 150.0, "r13": 250.0, "angle_param": "mu",
        "mu": {"mu_min": -0.8, "mu_max": 0.8, "n_mu": 3}, "n_rot": 3, "center": "particle", "base_seed": 9,
        "weight_normalization": "field", "products": ["zeta", "ddd"]}}, device="cpu").run()
    for k in ("ddd", "d_delta_dd", "rrr", "xi23", "r_delta_dd", "delta_ddd", "zeta"):
        ref = g["p3_" + k]
        assert np.abs(getattr(d, k) - ref).max() <= 1e-5 * np.abs(ref).max(), (k, getattr(d, k), ref)


def test_catalogue_path_resolution(tmp_path):
    """resolve_data_path (io/resources.py:87-160) as read_particle_data
    uses it: SHA256 checks on local files, the deterministic cache path of
    an http(s) catalogue, reuse of a cached copy without the network, and a
    clear error for a catalogue that would need downloading."""
    from pyhermes_gb300 import resources as rs

    pos = np.arange(12, dtype=np.float32).reshape(4, 3)
    local = tmp_path / "cat.bin"
    pos.tofile(local)
    digest = rs.file_sha256(local)
    assert len(digest) == 64
    d = read_particle_data(str(local), "bin", download={"sha256": "sha256:" + digest.upper()})
    assert np.array_equal(d["pos"], pos)
    with pytest.raises(ValueError, match="SHA256 mismatch"):
        read_particle_data(str(local), "bin", download={"sha256": "0" * 64})
    with pytest.raises(ValueError, match="64-character"):
        read_particle_data(str(local), "bin", download={"sha256": "abc"})
    url = "https://example.invalid/data/cat%201.bin"
    assert rs.is_remote_url(url) and not rs.is_remote_url(str(local)) and not rs.is_remote_url(3)
    target = rs.remote_cache_path(url, cache_dir=tmp_path / "cache")
    assert target.name.endswith("-cat 1.bin") and len(target.name.split("-")[0]) == 12
    with pytest.raises(ValueError, match="not in the cache"):
        read_particle_data(url, "bin", download={"cache_dir": str(tmp_path / "cache")})
    target.parent.mkdir(parents=True)
    pos.tofile(target)
    d = read_particle_data(url, "bin", download={"cache_dir": str(tmp_path / "cache"), "sha256": digest})
    assert np.array_equal(d["pos"], pos)
    with pytest.raises(ValueError, match="Set only one"):
        rs.resolve_data_path(url, cache_path=str(target), cache_dir=str(tmp_path))
