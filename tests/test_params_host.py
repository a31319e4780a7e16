"""Host-side parameter handling (no GPU): the parameter copy used on the
per-bin window paths behaves as copy.deepcopy, and the (s, mu) -> (R, H)
binning windows carry the reference mapping (corr2pcf.py mapping_smu_to_RH)."""
import copy

import numpy as np
import pytest

from pyhermes_gb300.corr2pcf import build_binning_window_params_for_sample, normalize_binning_window
from pyhermes_gb300.params import plain_copy


def test_plain_copy_matches_deepcopy():
    def f(k):
        return k

    src = {"type": "ring", "len_args": {"R": None, "H": 2.5}, "los_args": {"nx": 0.0, "ny": 0.0, "nz": 1.0},
           "other_args": {"table": np.arange(4.0), "func": f, "nested": [1, (2, {"a": 3})]}, "mapping": "smu_to_RH"}
    a, b = plain_copy(src), copy.deepcopy(src)
    assert a.keys() == b.keys()
    assert a["len_args"] == b["len_args"] and a["los_args"] == b["los_args"]
    assert a["other_args"]["nested"] == b["other_args"]["nested"]
    np.testing.assert_array_equal(a["other_args"]["table"], src["other_args"]["table"])
    # no aliasing of containers or arrays; functions are shared, as deepcopy does
    assert a["len_args"] is not src["len_args"] and a["other_args"]["nested"][1][1] is not src["other_args"]["nested"][1][1]
    assert a["other_args"]["table"] is not src["other_args"]["table"]
    assert a["other_args"]["func"] is f and b["other_args"]["func"] is f
    a["len_args"]["R"] = 1.0
    a["other_args"]["table"][0] = 9.0
    assert src["len_args"]["R"] is None and src["other_args"]["table"][0] == 0.0


def test_ring_binning_params_per_sample_are_independent():
    bw = normalize_binning_window({"type": "ring"})
    before = copy.deepcopy(bw)
    p1 = build_binning_window_params_for_sample({"s": 50.0, "mu": 0.6}, bw)
    p2 = build_binning_window_params_for_sample({"s": 20.0, "mu": 0.0}, bw)
    assert np.isclose(p1["len_args"]["R"], 50.0 * np.sqrt(1 - 0.36)) and np.isclose(p1["len_args"]["H"], 30.0)
    assert p2["len_args"]["R"] == 20.0 and p2["len_args"]["H"] == 0.0
    assert "mapping" not in p1 and p1["len_args"] is not p2["len_args"]
    assert bw == before  # the task's template is untouched


def test_window_defaults_are_not_shared():
    """Each window default is its own dict: merging one vertex's len_args
    must not reach another's."""
    from pyhermes_gb300.params import task_params

    for task in ("Corr_2PCF", "Corr_3PCF", "Corr_3PCF_Multipole"):
        tp = task_params(task, {task: {"window1": {"type": "gaussian", "len_args": {"R": 40.0}},
                                       "window2": {"type": "sphere", "len_args": {"R": 60.0}}}})
        assert tp["window1"]["len_args"] == {"R": 40.0} and tp["window2"]["len_args"] == {"R": 60.0}
        assert tp["window"]["len_args"] == {}


def test_reference_import_paths():
    """The reference's import paths (pyhermes.theory / .base / .io) exist
    under this package and name the same objects."""
    from pyhermes_gb300 import corr2pcf, counting, mc3pcf, multipole, projection, sfc_field, window
    from pyhermes_gb300.base import SFCProjection as P2, WindowFunc as W2
    from pyhermes_gb300.io import (Corr2PCFData, Corr3PCFData, Corr3PCFMultipoleData, CountingData, SFCField,
                                   WindowFunc, check_fout)
    from pyhermes_gb300.theory import Corr_2PCF, Corr_3PCF, Corr_3PCF_Multipole, Counting, SFCProjection

    assert (Corr_2PCF, Corr_3PCF, Corr_3PCF_Multipole, Counting) == (
        corr2pcf.Corr_2PCF, mc3pcf.Corr_3PCF, multipole.Corr_3PCF_Multipole, counting.Counting)
    assert SFCProjection is P2 is projection.SFCProjection and WindowFunc is W2 is window.WindowFunc
    assert SFCField is sfc_field.SFCField and check_fout is sfc_field.check_fout
    assert (Corr2PCFData, Corr3PCFData, Corr3PCFMultipoleData, CountingData) == (
        corr2pcf.Corr2PCFData, mc3pcf.Corr3PCFData, multipole.Corr3PCFMultipoleData, counting.CountingData)


def test_multipole_binning_template_rules():
    """theory/corr3pcf_multipole.py:205-227, 296-324: template checks and
    mapping targets."""
    from pyhermes_gb300.multipole import Corr_3PCF_Multipole

    def task(bw12, sampling=None):
        return Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
            "binning_window12": bw12,
            "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
            "sampling": sampling or {"mode": "paired", "r12": [100.0], "r13": [200.0]},
            "l_min": 0, "l_max": 1}}, device="cpu")

    t = task({"type": " Thick_Shell ", "len_args": None, "other_args": None,
              "mapping": {"R": "r12", "len_args.delta_R": 40.0, "other_args.x": "r13"}})
    w = t.binning_window12[0]
    assert w["type"] == "thick_shell" and w["len_args"] == {"R": 100.0, "delta_R": 40.0}
    assert w["other_args"] == {"x": 200.0} and "mapping" not in w
    assert t.binning_window12_template["type"] == "thick_shell"
    with pytest.raises(ValueError, match="non-empty 'type'"):
        task({"type": "", "mapping": {"R": "r12"}})
    with pytest.raises(TypeError, match="mapping must be a dictionary"):
        task({"type": "shell", "mapping": [("R", "r12")]})
    with pytest.raises(KeyError, match="not defined"):
        task({"type": "shell", "mapping": {"R": "s"}})
    with pytest.raises(ValueError, match="Unsupported binning-window mapping target"):
        task({"type": "shell", "mapping": {"R": "r12", "los_args.nx": 1.0}})
    with pytest.raises(ValueError, match="empty len_args"):
        task({"type": "shell", "mapping": {}})


def test_format_params_rereads_task_params():
    """Task.format_params (theory/*.py format_params) re-reads task_params."""
    from pyhermes_gb300.corr2pcf import Corr_2PCF
    from pyhermes_gb300.mc3pcf import Corr_3PCF
    from pyhermes_gb300.multipole import Corr_3PCF_Multipole

    t = Corr_2PCF({"Corr_2PCF": {"random": "uniform"}}, device="cpu")
    t.task_params["random2"] = "r.pkl"
    t.format_params()
    assert (t.random1, t.random2) == ("uniform", "r.pkl")
    m = Corr_3PCF({"Corr_3PCF": {"r12": 10.0}}, device="cpu")
    m.task_params["r13"] = 55.0
    m.format_params()
    assert (m.r12, m.r13) == (10.0, 55.0)
    q = Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "binning_window12": {"type": "shell", "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [100.0], "r13": [200.0]}}}, device="cpu")
    q.task_params["l_max"] = 6
    q.format_params()
    assert q.l_max == 6
