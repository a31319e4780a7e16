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


WIN_CODES = {
    "sphere": 0, "gaussian": 1, "shell": 2, "thick_shell": 3, "gaussian_shell": 4, "cubic": 5,
    "ring": 6, "disk": 7, "cylshell": 8, "cylinder": 9, "cw": 10, "cws": 11, "gdw": 12,
    "directional_derivative": 13, "laplacian": 14, "inverse_laplacian": 15,
}
WIN_ARGS = {
    "sphere": ("R",), "gaussian": ("R",), "shell": ("R",), "thick_shell": ("R", "delta_R"),
    "gaussian_shell": ("R_shell", "R_smooth"), "cubic": ("Lx", "Ly", "Lz"),
    "ring": ("R", "H"), "disk": ("R", "H"), "cylshell": ("R", "H"), "cylinder": ("R", "H"),
    "cw": ("R",), "cws": ("R",), "gdw": ("R",), "directional_derivative": (),
    "laplacian": (), "inverse_laplacian": (),
}


def fourier_power(phi, k_max, k_count, res=1024):
    """utils/wavelet_grid.py:94-118: |phi_hat|^2 by direct DFT (float64)."""
    phi = np.asarray(phi, dtype=np.float64)
    n = phi.shape[0]
    dx = (n / res) / n
    k = np.arange(k_count + 1) * (k_max / k_count)
    x = np.arange(n) * dx
    arg = (-2 * np.pi * k)[:, None] * x[None, :]
    re = np.sum(phi * dx * np.cos(arg), axis=1)
    im = np.sum(phi * dx * np.sin(arg), axis=1)
    return re ** 2 + im ** 2


def window_kernel(wtype, len_args, L, P, mode="octant", los=(0.0, 0.0, 1.0), bandwidth=1, box=1000.0):
    """The reference WindowFunc kernel (io/window.py:274-332) in float64.

    len_args are physical lengths (rescaled here by L/box like io/window.py:112).
    mode: 'octant' (convolution.py:14-38 + 263-281), 'full_rfft' (:73-157) or
    'complex_rfft' (:168-252).  Returns [L, L, L/2+1] real or complex."""
    args = np.zeros(4)
    for i, nm in enumerate(WIN_ARGS[wtype]):
        args[i] = float(len_args[nm]) * L / box
    los = np.ascontiguousarray(los, dtype=np.float64)
    P = np.ascontiguousarray(P, dtype=np.float64)
    H = L // 2 + 1
    code = WIN_CODES[wtype]
    lb = lib()
    lb.oracle_window_octant.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lb.oracle_window_rfft.argtypes = lb.oracle_window_octant.argtypes
    if mode == "octant":
        out = np.empty((L, L, H), dtype=np.float64)
        lb.oracle_window_octant(code, _p(args), _p(los), L, bandwidth, _p(P), _p(out))
    else:
        out2 = np.empty((L, L, H, 2), dtype=np.float64)
        lb.oracle_window_rfft(code, _p(args), _p(los), L, bandwidth, _p(P), _p(out2))
        out = out2[..., 0] + 1j * out2[..., 1] if mode == "complex_rfft" else out2[..., 0].copy()
    if wtype == "inverse_laplacian":
        out[0, 0, 0] = 0.0
    return out


def convolve(eps, kernel):
    """utils/convolution.py:284-288: irfftn(rfftn(eps) * K)."""
    from scipy.fft import irfftn, rfftn

    sc = rfftn(np.asarray(eps, dtype=np.float64))
    sc *= kernel
    return irfftn(sc, s=eps.shape)


def pair_product(eps1, eps2, kernel):
    """theory/corr2pcf.py:366-372: mean((eps1 conv K) * eps2)."""
    conv = convolve(eps1, kernel)
    return float(np.einsum("ijk,ijk->", conv, eps2, optimize=True) / conv.size)
