"""WindowFunc composite algebra against the reference (no GPU): kernels of
window +, -, x with windows and scalars (nested), and the file a composite
window saves (golden composite_windows_J4.npz).  The component kernels come
from the oracle's kernel builder on the CPU."""
import json
import os

import numpy as np
import pytest
import torch

import oracle
from pyhermes_gb300 import window as win_mod
from pyhermes_gb300.phi import sample_scaling_function
from pyhermes_gb300.sfc_field import read_numpy_pickle
from pyhermes_gb300.window import WindowFunc
from test_field_algebra_host import _clean, _close

PHI = sample_scaling_function()
SFC = {"J": 4, "box_size": 1000.0, "phi_resolution": 1024, "wavelet_mode": "db2", "wavelet_level": 10}


@pytest.fixture
def cpu_windows(monkeypatch):
    orig = WindowFunc.kernel_device

    def kernel_device(self):
        if self.is_composite_window:
            return orig(self)
        K = oracle.window_kernel(self.type, self.len_args, self.L, oracle.fourier_power(PHI, self.bandwidth, self.L),
                                 mode=self.resolved_mode(), box=self.box_size)
        return torch.as_tensor(K)

    monkeypatch.setattr(WindowFunc, "kernel_device", kernel_device)


def test_composite_window_kernels_match_reference(golden_dir, cpu_windows, tmp_path):
    g = np.load(os.path.join(golden_dir, "composite_windows_J4.npz"))
    a = WindowFunc({"type": "gaussian", "len_args": {"R": 30.0}}, SFC, device="cpu")
    b = WindowFunc({"type": "sphere", "len_args": {"R": 50.0}}, SFC, device="cpu")
    for name, w in {"add": a + b, "sub": a - 0.5 * b, "neg": -a, "prod": a * b, "div": a / 4.0,
                    "nested": (a + b) * 2.0 - a}.items():
        ref = g[name + "_kernel"]
        got = np.asarray(w.as_array())
        assert got.shape == ref.shape and np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), name
    c = a + b
    c.save(str(tmp_path / "w.pkl"))
    with open(tmp_path / "w.pkl", "rb") as f:
        d = read_numpy_pickle(f)
    assert list(d.keys()) == [str(k) for k in g["saved_keys"]]
    _close(_clean({k: v for k, v in d.items() if k != "window_kernal"}), json.loads(str(g["saved_info"])), "saved")
    assert np.abs(np.asarray(d["window_kernal"]) - g["saved_kernel"]).max() <= 1e-12 * np.abs(g["saved_kernel"]).max()
    with pytest.raises((ZeroDivisionError, ValueError)):
        a / 0.0
