"""WindowFunc files in the reference's framed-pickle format: the reference's
own saved window (tests/golden/window_gaussian_J4.pkl, written by
make_golden.py) reads here, and a window saved here carries the same keys
and kernel."""
import os

import numpy as np
import pytest

from pyhermes_gb300.sfc_field import read_numpy_pickle

SFC = {"J": 4, "box_size": 1000.0, "phi_resolution": 1024, "wavelet_mode": "db2", "wavelet_level": 10}


def test_reference_window_file_reads(golden_dir):
    with open(os.path.join(golden_dir, "window_gaussian_J4.pkl"), "rb") as f:
        d = read_numpy_pickle(f)
    assert d["type"] == "gaussian" and d["len_args"] == {"R": 90.0}
    g = np.load(os.path.join(golden_dir, "window_file_J4.npz"))
    np.testing.assert_array_equal(d["window_kernal"], g["kernel"])


@pytest.mark.gpu
def test_window_save_load_round_trip(golden_dir, tmp_path):
    import torch

    from pyhermes_gb300.window import WindowFunc

    ref_path = os.path.join(golden_dir, "window_gaussian_J4.pkl")
    w = WindowFunc({"type": "gaussian", "len_args": {"R": 90.0}}, SFC)
    out = str(tmp_path / "w.pkl")
    w.save(out)
    with open(out, "rb") as f:
        mine = read_numpy_pickle(f)
    with open(ref_path, "rb") as f:
        ref = read_numpy_pickle(f)
    assert set(mine) >= {"type", "len_args", "J", "box_size", "window_kernal"}
    k_ref = ref["window_kernal"]
    assert np.abs(mine["window_kernal"] - k_ref).max() < 1e-6 * np.abs(k_ref).max()
    back = WindowFunc({"type": "gaussian", "len_args": {"R": 10.0}}, SFC)
    back.load(ref_path)
    assert back.input_params["len_args"] == {"R": 90.0}
    np.testing.assert_allclose(back.kernel_device().double().cpu().numpy(), k_ref, rtol=1e-6, atol=1e-7)
    from pyhermes_gb300.sfc_field import SFCField

    f = SFCField(device="cuda")
    f.sfc_info = dict(SFC, L=16, V=16 ** 3, scale_factor=16 / 1000.0, phi_support=3, field_kind="derived_field")
    f.format_sfc_params()
    f.epsilon_device = torch.randn((16, 16, 16), device="cuda", dtype=torch.float32)
    a = (f @ w).epsilon_device
    b = (f @ back).epsilon_device
    assert float((a - b).abs().max() / a.abs().max()) < 1e-5
