"""Result and field files against files written by the reference's own save
methods (tests/golden/io, NumPy-framed pickles): the reference's files load
through this package's loaders, and the files this package writes have the
reference's top-level keys in the reference's order, the same info keys and
the same values (tasks run on the CPU with the oracle kernels)."""
import os

import numpy as np
import pytest
import torch

from pyhermes_gb300 import corr2pcf, mc3pcf
from pyhermes_gb300 import multipole as mp
from pyhermes_gb300.counting import Counting, CountingData
from pyhermes_gb300.projection import SFCProjection
from pyhermes_gb300.sfc_field import SFCField, read_numpy_pickle
from test_tasks_host import _cpu_triplet_sum, oracle_kernels  # noqa: F401  (fixture)


def _read(path):
    with open(path, "rb") as f:
        return read_numpy_pickle(f)


def _io(golden_dir, name):
    return os.path.join(golden_dir, "io", name)


def _field(golden_dir):
    cat = np.load(_io(golden_dir, "catalogue.npz"))
    return SFCProjection({"SFCProjection": {"particle_pos": cat["pos"], "catalog_weight": cat["weights"], "J": 4,
                                            "box_size": 1000.0}}, device="cpu").run(save_result=False)


def _rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / np.abs(b).max()


def _same_layout(ours, ref, info_key=None):
    assert list(ours) == list(ref), (list(ours), list(ref))
    if info_key:
        assert set(ours[info_key]) == set(ref[info_key]), (set(ours[info_key]) ^ set(ref[info_key]))


@pytest.fixture
def cpu_mc(monkeypatch):
    monkeypatch.setattr(mc3pcf, "triplet_sum", _cpu_triplet_sum)

    def interp(grid, J, scaled_pos, phi_t, offset=(0.0, 0.0, 0.0)):
        import oracle

        p = scaled_pos.cpu().numpy() if isinstance(scaled_pos, torch.Tensor) else np.asarray(scaled_pos)
        return torch.as_tensor(oracle.interp(p, grid.double().cpu().numpy(), phi_t.double().cpu().numpy(), J,
                                             offset=offset))

    monkeypatch.setattr(mc3pcf, "interp", interp)


def test_sfc_field_file(golden_dir, oracle_kernels, tmp_path):
    ref = _read(_io(golden_dir, "field_J4.pkl"))
    f = SFCField(data_path=_io(golden_dir, "field_J4.pkl"), device="cpu")
    np.testing.assert_array_equal(f.epsilon, ref["epsilon"])
    assert f.sfc_info["field_integral"] == ref["sfc_info"]["field_integral"]
    ours = _field(golden_dir)
    ours.save_sfc_field(str(tmp_path / "f.pkl"))
    d = _read(str(tmp_path / "f.pkl"))
    _same_layout(d, ref, "sfc_info")
    assert np.abs(d["epsilon"] - ref["epsilon"]).max() <= 2e-6 * np.abs(ref["epsilon"]).max()


def test_corr2pcf_file(golden_dir, oracle_kernels, tmp_path):
    ref = _read(_io(golden_dir, "corr2pcf_J4.pkl"))
    got = corr2pcf.Corr2PCFData(data_path=_io(golden_dir, "corr2pcf_J4.pkl"))
    np.testing.assert_array_equal(got.xi, ref["xi"])
    np.testing.assert_array_equal(got.s, ref["s"])
    out = str(tmp_path / "c2.pkl")
    corr2pcf.Corr_2PCF({"Corr_2PCF": {
        "sfc_field": _field(golden_dir), "random": "uniform", "fout_path": out,
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": 60.0}, "mapping": "s_to_R"},
        "sampling": {"s": {"min": 100.0, "max": 300.0, "n": 3}}, "products": ["dd", "xi"]}}, device="cpu").run()
    d = _read(out)
    _same_layout(d, ref, "corr2pcf_info")
    for k in ("dd", "delta_dd", "rr", "xi", "s"):
        assert _rel(d[k], ref[k]) < 1e-5, k
    assert d["dr"] is None and ref["dr"] is None


def test_counting_file(golden_dir, oracle_kernels, cpu_mc, tmp_path):
    ref = _read(_io(golden_dir, "counting_J4.pkl"))
    got = CountingData(data_path=_io(golden_dir, "counting_J4.pkl"))
    np.testing.assert_array_equal(got.nx, ref["nx"])
    out = str(tmp_path / "n.pkl")
    Counting({"Counting": {"sfc_field": _field(golden_dir), "random_count": 50, "seed": 3, "fout_path": out}},
             device="cpu").run()
    d = _read(out)
    _same_layout(d, ref, "counting_info")
    assert _rel(d["nx"], ref["nx"]) < 1e-5


def test_corr3pcf_file(golden_dir, oracle_kernels, cpu_mc, tmp_path):
    ref = _read(_io(golden_dir, "corr3pcf_J4.pkl"))
    got = mc3pcf.Corr3PCFData(data_path=_io(golden_dir, "corr3pcf_J4.pkl"))
    np.testing.assert_array_equal(got.zeta, ref["zeta"])
    out = str(tmp_path / "c3.pkl")
    mc3pcf.Corr_3PCF({"Corr_3PCF": {
        "sfc_field": _field(golden_dir), "random": "uniform", "r12": 150.0, "r13": 250.0, "angle_param": "mu",
        "mu": {"mu_min": -0.5, "mu_max": 0.5, "n_mu": 2}, "n_rot": 2, "center": "box_random",
        "n_box_centers": 100, "base_seed": 42, "products": ["zeta", "ddd"], "fout_path": out}}, device="cpu").run()
    d = _read(out)
    _same_layout(d, ref, "corr3pcf_info")
    for k in ("mu", "theta", "r23", "ddd", "rrr", "delta_ddd", "xi23", "zeta"):
        assert _rel(d[k], ref[k]) < 1e-5, k


def test_corr3pcf_multipole_file(golden_dir, oracle_kernels, tmp_path):
    ref = _read(_io(golden_dir, "corr3pcf_multipole_J4.pkl"))
    got = mp.Corr3PCFMultipoleData(data_path=_io(golden_dir, "corr3pcf_multipole_J4.pkl"))
    np.testing.assert_array_equal(got.zeta_l, ref["zeta_l"])
    out = str(tmp_path / "m.pkl")
    mp.Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field": _field(golden_dir), "random": "uniform", "fout_path": out,
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [150.0], "r13": [250.0]},
        "l_min": 0, "l_max": 1, "summation_backend": "cpu", "products": ["ddd_l", "zeta_l"]}}, device="cpu").run()
    d = _read(out)
    _same_layout(d, ref, "corr3pcf_multipole_info")
    for k in ("ddd_l", "delta_ddd_l", "rrr_l", "zeta_l"):
        assert _rel(d[k], ref[k]) < 1e-5, k


def test_output_path_rules(golden_dir, tmp_path, oracle_kernels):
    """check_fout (io/funcs.py:13-57) as every saver applies it: no path
    writes nothing, an existing file gets the next free name_<n> unless
    overwrite, a folder receives Output_<Class>_<stamp>.pkl, and the generic
    save / load flags of io/base.py:24-124 reach the field writer."""
    import re

    f = _field(golden_dir)
    assert f.save_sfc_field("") is None and f.save_sfc_field(None) is None
    first = f.save_sfc_field(str(tmp_path / "a" / "f.pkl"))
    assert first == str(tmp_path / "a" / "f.pkl") and os.path.isfile(first)
    assert f.save_sfc_field(first) == str(tmp_path / "a" / "f_1.pkl")
    assert f.save(first, save_sfc_field=True) == str(tmp_path / "a" / "f_2.pkl")
    assert f.save_sfc_field(first, overwrite=True) == first
    out = f.save_sfc_field(str(tmp_path / "dir") + os.sep)
    assert re.fullmatch(r"Output_SFCField_\d{12}\.pkl", os.path.basename(out)) and os.path.isfile(out)
    g = SFCField(device="cpu")
    g.sfc_info = {}
    g.load(first, read_sfc_field=True)
    assert np.array_equal(g.epsilon, f.epsilon)
    with pytest.raises(ValueError):
        f.save(first, save_2pcf=True)
    d = CountingData()
    d.counting_info, d.sfc_info, d.nx = {"seed": 1}, dict(f.sfc_info), np.arange(3.0)
    p = d.save_counting(str(tmp_path / "c.pkl"))
    assert d.save_counting(p) == str(tmp_path / "c_1.pkl")


def test_result_containers_generic_save_load(tmp_path):
    """io/base.py:24-124 on the result containers: save(..., save_2pcf=True)
    / load(..., read_2pcf=True) and the flagless forms write and read the
    container's own file; another kind's flag is refused."""
    d = corr2pcf.Corr2PCFData()
    d.set_sampling(("s",), {"s": np.array([1.0, 2.0])})
    d.dd = np.array([3.0, 4.0])
    d.corr2pcf_info = {"k": 1}
    p1 = d.save(str(tmp_path / "c2.pkl"), save_2pcf=True)
    p2 = d.save(str(tmp_path / "c2.pkl"))
    assert p2.endswith("c2_1.pkl")
    for p, kw in ((p1, {"read_2pcf": True}), (p2, {})):
        e = corr2pcf.Corr2PCFData()
        e.load(p, **kw)
        assert np.array_equal(e.dd, d.dd) and np.array_equal(e.s, d.s)
    with pytest.raises(ValueError):
        d.save(str(tmp_path / "x.pkl"), save_counting=True)
    with pytest.raises(ValueError):
        corr2pcf.Corr2PCFData().load(p1, read_3pcf=True)
    c = CountingData()
    c.counting_info, c.sfc_info, c.nx = {"seed": 1}, {"J": 4}, np.arange(3.0)
    q = c.save(str(tmp_path / "n.pkl"), save_counting=True)
    c2 = CountingData()
    c2.load(q, read_counting=True)
    assert np.array_equal(c2.nx, c.nx)
