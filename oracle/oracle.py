"""Oracle: float64 CPU restatement of the PyHermes field pipeline.

TEST INFRASTRUCTURE ONLY.  tests/, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` use it as the checker; the product package
(``pyhermes_gb300``) never imports it.

The hot loops live in ``hermes_oracle.c`` (built by ``oracle/build_oracle.py``
into ``oracle/_build/libhermes_oracle.so``); FFTs use scipy.fft (pocketfft),
the same library the reference calls (``pyhermes/utils/convolution.py:7``).
Every function cites the reference lines it restates.
"""

import ctypes
import os

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        from build_oracle import build  # noqa: E402  (sibling module)

        path = build()
        _LIB = ctypes.CDLL(path)
        P = ctypes.c_void_p
        I64 = ctypes.c_int64
        I = ctypes.c_int
        D = ctypes.c_double
        _LIB.oracle_deposit.argtypes = [P, P, I64, P, I, I, I, D, P]
        _LIB.oracle_cell_counts.argtypes = [P, I64, I, D, P]
        _LIB.oracle_interp.argtypes = [P, I64, P, I, P, I, I, D, D, D, P]
        _LIB.oracle_num_threads.restype = I
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def num_threads():
    return int(lib().oracle_num_threads())


def deposit(pos, w, phi, J, box, res=1024):
    """utils/wavelet_grid.py:58-70 project_scaling_grid_numba -> float64 [L,L,L]."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    L = 1 << J
    grid = np.empty((L, L, L), dtype=np.float64)
    lib().oracle_deposit(_p(pos), _p(w), pos.shape[0], _p(phi), phi.size, res, J, float(box), _p(grid))
    return grid


def cell_counts(pos, J, box):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    L = 1 << J
    out = np.empty((L, L, L), dtype=np.uint32)
    lib().oracle_cell_counts(_p(pos), pos.shape[0], J, float(box), _p(out))
    return out


def interp(scaled_pos, grid, phi, J, res=1024, offset=(0.0, 0.0, 0.0)):
    """utils/wavelet_grid.py:143-186 interpolate_grid_at_pos_numba."""
    scaled_pos = np.ascontiguousarray(scaled_pos, dtype=np.float64)
    grid = np.ascontiguousarray(grid, dtype=np.float64)
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    out = np.empty(scaled_pos.shape[0], dtype=np.float64)
    lib().oracle_interp(_p(scaled_pos), scaled_pos.shape[0], _p(grid), J, _p(phi), phi.size, res,
                        float(offset[0]), float(offset[1]), float(offset[2]), _p(out))
    return out


def projection_weights(catalog_weight, field_value, mode="catalog"):
    """base/sfc_projection.py:251-282: float64 p_w = w*q/denominator."""
    cw = np.asarray(catalog_weight, dtype=np.float64)
    fv = np.asarray(field_value, dtype=np.float64)
    cw_sum = float(np.sum(cw, dtype=np.float64))
    raw = float(np.sum(cw * fv, dtype=np.float64))
    if mode == "raw":
        den = 1.0
    elif mode == "catalog":
        den = cw_sum
    else:
        den = raw
    return cw * fv / den, raw / den
