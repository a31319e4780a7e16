"""SFCField algebra and normalisation against the reference (no GPU): the
epsilon and sfc_info of field +, -, *, / with fields and scalars, weight
normalisation switches and unit weights, mean densities and
field_density_at_pos for every normalisation and value unit
(golden field_algebra_J4.npz; fields projected on the CPU with the oracle
deposit, read as float32 as on the GPU)."""
import json
import os

import numpy as np
import pytest
import torch

import oracle
from pyhermes_gb300 import mc3pcf
from pyhermes_gb300.projection import SFCProjection
from test_tasks_host import oracle_kernels  # noqa: F401  (fixture)

OPS = ("add", "sub", "mul", "adds", "subs", "rsubs", "muls", "divs", "switch_raw", "switch_field", "unit", "with_raw")


def _clean(v):
    if isinstance(v, dict):
        return {k: _clean(x) for k, x in v.items() if k != "phi_array"}
    if isinstance(v, (list, tuple)):
        return [_clean(x) for x in v]
    if isinstance(v, (np.floating, np.integer)):
        return v.item()
    if isinstance(v, np.ndarray):
        return v.tolist()
    return v


def _close(a, b, path=""):
    if isinstance(b, dict):
        assert isinstance(a, dict) and set(a) == set(b), (path, set(a) ^ set(b) if isinstance(a, dict) else a)
        for k in b:
            _close(a[k], b[k], f"{path}.{k}")
    elif isinstance(b, list):
        assert isinstance(a, list) and len(a) == len(b), (path, a, b)
        for i, (x, y) in enumerate(zip(a, b)):
            _close(x, y, f"{path}[{i}]")
    elif isinstance(b, float) and not isinstance(a, bool):
        assert a is not None and abs(a - b) <= 1e-6 * max(1e-300, abs(b)), (path, a, b)
    else:
        assert a == b, (path, a, b)


@pytest.fixture
def fields(golden_dir, oracle_kernels, monkeypatch):
    def interp(grid, J, scaled_pos, phi_t, offset=(0.0, 0.0, 0.0)):
        p = scaled_pos.cpu().numpy() if isinstance(scaled_pos, torch.Tensor) else np.asarray(scaled_pos)
        return torch.as_tensor(oracle.interp(p, grid.double().cpu().numpy(), phi_t.double().cpu().numpy(), J,
                                             offset=offset))

    monkeypatch.setattr(mc3pcf, "interp", interp)
    g = np.load(os.path.join(golden_dir, "field_algebra_J4.npz"))
    a = SFCProjection({"SFCProjection": {"particle_pos": g["pa"], "catalog_weight": g["wa"],
                                         "field_value": g["fva"], "J": 4, "box_size": 1000.0}},
                      device="cpu").run(save_result=False)
    b = SFCProjection({"SFCProjection": {"particle_pos": g["pb"], "J": 4, "box_size": 1000.0}},
                      device="cpu").run(save_result=False)
    return g, a, b


@pytest.mark.parametrize("op", OPS)
def test_field_algebra_matches_reference(fields, op):
    g, a, b = fields
    r = {"add": lambda: a + b, "sub": lambda: a - b, "mul": lambda: a * b, "adds": lambda: a + 0.5,
         "subs": lambda: a - 0.25, "rsubs": lambda: 1.0 - a, "muls": lambda: 3.0 * a, "divs": lambda: a / 4.0,
         "switch_raw": lambda: a.switch_weight_normalization("raw"),
         "switch_field": lambda: a.switch_weight_normalization("field"), "unit": lambda: a.to_unit_weight(),
         "with_raw": lambda: a.with_normalization("raw")}[op]()
    ref = g[op + "_eps"]
    assert np.abs(np.asarray(r.epsilon) - ref).max() <= 2e-6 * np.abs(ref).max(), op
    _close(_clean(r.sfc_info), json.loads(str(g[op + "_info"])), op)


def test_mean_density_and_density_at_pos_match_reference(fields):
    g, a, _ = fields
    means = json.loads(str(g["means"]))
    for norm in (None, "raw", "field", "unit"):
        for unit in ("grid", "physical"):
            key = f"{norm}_{unit}"
            m = a.field_mean_density(normalization=norm, value_unit=unit)
            assert abs(m - means["mean_" + key]) <= 1e-12 * abs(means["mean_" + key]), (key, m)
            got = np.asarray(a.field_density_at_pos(g["query"], normalization=norm, value_unit=unit))
            ref = g["at_" + key]
            assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max(), key


def test_phi_at_pos_matches_reference(golden_dir, oracle_kernels):
    """SFCField.phi_at_pos (io/sfc_field.py:484-485): cells and stencils
    bit-identical to the reference, boundary positions included."""
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "phi_at_pos_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "J": 4, "box_size": 1000.0}},
                      device="cpu").run(save_result=False)
    coarse, local = f.phi_at_pos(g["pos"])
    assert coarse.dtype == np.int32 and np.array_equal(coarse, g["coarse"])
    assert local.shape == (200, 3, 3, 3) and np.array_equal(local, g["local"])
