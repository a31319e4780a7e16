"""Corr_2PCF bins of one built-in window family: the per-bin descriptors
built from one template (window.family_descriptors) are byte-identical to
the descriptors of one WindowFunc per bin, for the reference's mappings
(s -> R, (s, mu) -> (R, H), (r_p, pi) -> (R, H)) and several window types;
sampling whose bins differ in more than lengths falls back to per-bin
windows."""
import ctypes

import numpy as np
import pytest

from pyhermes_gb300 import corr2pcf
from pyhermes_gb300.window import HermesWindow, WindowFunc

SFC = {"J": 6, "L": 64, "box_size": 1000.0, "phi_resolution": 1024, "wavelet_mode": "db2", "wavelet_level": 10}


def _task(bw, sampling):
    t = corr2pcf.Corr_2PCF.__new__(corr2pcf.Corr_2PCF)
    t.binning_window = corr2pcf.normalize_binning_window(bw)
    t.sampling_names = list(sampling)
    t.sampling_arrays = {n: np.asarray(v, dtype=np.float64) for n, v in sampling.items()}
    t.threads = 1
    t.device = "cpu"
    return t


class _Ref:
    sfc_info = dict(SFC)


@pytest.mark.parametrize("bw,sampling", [
    ({"type": "ring"}, {"s": np.linspace(7.0, 145.0, 12), "mu": np.linspace(0.05, 0.95, 5)}),
    ({"type": "thick_shell", "len_args": {"delta_R": 7.25}}, {"s": np.linspace(8.0, 140.0, 9)}),
    ({"type": "cylinder", "mapping": "rppi_to_RH"}, {"rp": np.linspace(5.0, 60.0, 4), "pi": np.linspace(5.0, 80.0, 3)}),
    ({"type": "shell"}, {"s": [10.0, 20.0, 40.0]}),
])
def test_family_descriptors_equal_per_bin_windows(bw, sampling):
    task = _task(bw, sampling)
    fam = task._binning_family(_Ref())
    assert fam is not None
    template, descs = fam
    wins = task._binning_windows(_Ref())
    assert len(descs) == len(wins)
    n = ctypes.sizeof(HermesWindow)
    for d, w in zip(descs, wins):
        assert ctypes.string_at(ctypes.addressof(d), n) == ctypes.string_at(ctypes.addressof(w.descriptor()), n)
