"""``WindowFunc`` and ``field @ window`` on the GPU.

Mirrors ``pyhermes/io/window.py:32-548`` and the parameter rules of
``pyhermes/utils/window_params.py``: the same ``win_params`` dicts, length
rescaling by L/box (:112), line-of-sight normalisation, kernel-mode
resolution (:144-195), the inverse-Laplacian zero-mode rule (:266-272) and
composite window algebra (:364-485).

The kernel of a built-in window is never materialised for a convolution:
``hermes_window_apply`` evaluates it on the fly between the forward and
inverse FFT.  ``as_array()`` materialises it on the device (and returns a
NumPy copy, like the reference) for users and for composite algebra.
"""

import copy
import ctypes
import inspect
import os

import numpy as np
import torch

from . import _lib
from .kernels import _ptr, _stream_ptr
from .params import plain_copy
from .phi import fourier_power_spectrum, sample_scaling_function
from .sfc_field import SFCField

WIN_CODES = {
    "sphere": 0, "gaussian": 1, "shell": 2, "thick_shell": 3, "gaussian_shell": 4, "cubic": 5,
    "ring": 6, "disk": 7, "cylshell": 8, "cylinder": 9, "cw": 10, "cws": 11, "gdw": 12,
    "directional_derivative": 13, "laplacian": 14, "inverse_laplacian": 15,
}
# positional arguments after (ki, kj, kk), window_functions.py:29-438
WIN_ARGS = {
    "sphere": ("R",), "gaussian": ("R",), "shell": ("R",), "thick_shell": ("R", "delta_R"),
    "gaussian_shell": ("R_shell", "R_smooth"), "cubic": ("Lx", "Ly", "Lz"),
    "ring": ("R", "H"), "disk": ("R", "H"), "cylshell": ("R", "H"), "cylinder": ("R", "H"),
    "cw": ("R",), "cws": ("R",), "gdw": ("R",), "directional_derivative": (),
    "laplacian": (), "inverse_laplacian": (),
}
KMODE = {"octant": 0, "full_rfft": 1, "complex_rfft": 2}

ANISOTROPIC_AUTO_WINDOW_TYPES = {"ring", "disk", "cylinder", "cylshell"}
COMPLEX_RFFT_WINDOW_TYPES = {"directional_derivative"}
COMPLEX_FULL_FFT_WINDOW_TYPES = {"legendre_multipole", "radial_multipole"}
VALID_KERNEL_MODES = {"auto", "octant", "full_rfft", "complex_rfft", "complex_full_fft"}
LOS_ARG_KEYS = ("nx", "ny", "nz")
DEFAULT_LOS_ARGS = {"nx": 0.0, "ny": 0.0, "nz": 1.0}
LOS_AWARE_WINDOW_TYPES = ANISOTROPIC_AUTO_WINDOW_TYPES | COMPLEX_RFFT_WINDOW_TYPES
ZERO_MODE_ZERO_WINDOW_TYPES = {"inverse_laplacian"}


class HermesWindow(ctypes.Structure):
    """ctypes mirror of ``hermes_window_t`` (include/hermes_gb300.h)."""

    _fields_ = [("type", ctypes.c_int32), ("kernel_mode", ctypes.c_int32),
                ("zero_mode_zero", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("len", ctypes.c_double * 4), ("los", ctypes.c_double * 3),
                ("scale", ctypes.c_double)]


def normalize_los_args(los_args, window_type=None):
    """utils/window_params.py:50-72."""
    if los_args is None:
        los_args = {}
    if isinstance(los_args, (list, tuple, np.ndarray)):
        arr = np.asarray(los_args, dtype=np.float64)
        if arr.shape != (3,):
            raise ValueError("los_args array must contain exactly three values: [nx, ny, nz].")
        los_args = {k: float(v) for k, v in zip(LOS_ARG_KEYS, arr)}
    elif isinstance(los_args, dict):
        los_args = plain_copy(los_args)
    else:
        raise TypeError("los_args must be a dict, length-3 array, or None.")
    if not los_args and window_type in LOS_AWARE_WINDOW_TYPES:
        los_args = plain_copy(DEFAULT_LOS_ARGS)
    if los_args:
        if not all(k in los_args for k in LOS_ARG_KEYS):
            raise ValueError("los_args must define nx, ny, and nz together.")
        los = np.array([los_args[k] for k in LOS_ARG_KEYS], dtype=np.float64)
        if np.linalg.norm(los) == 0.0:
            raise ValueError("los_args vector must be non-zero.")
        los_args = {k: float(los_args[k]) for k in LOS_ARG_KEYS}
    return los_args


def default_kernel_mode(window_type, has_custom_func=False):
    """utils/window_params.py:75-84."""
    if has_custom_func:
        return "full_rfft"
    if window_type in COMPLEX_FULL_FFT_WINDOW_TYPES:
        return "complex_full_fft"
    if window_type in COMPLEX_RFFT_WINDOW_TYPES:
        return "complex_rfft"
    if window_type in ANISOTROPIC_AUTO_WINDOW_TYPES:
        return "auto"
    return "octant"


def normalize_kernel_mode(kernel_mode):
    mode = str(kernel_mode).strip().lower()
    if mode not in VALID_KERNEL_MODES:
        raise ValueError(f"Unsupported kernel_mode '{mode}'. Supported values are {sorted(VALID_KERNEL_MODES)}.")
    return mode


def ordered_window_args(func, kwargs):
    """Values of ``func``'s parameters after (kx, ky, kz), taken from
    ``kwargs`` or the parameter's default (utils/convolution.py:41-62)."""
    params = inspect.signature(func).parameters
    names = list(params)[3:]
    missing = [n for n in names if n not in kwargs and params[n].default is inspect.Parameter.empty]
    if missing:
        raise ValueError(f"Missing keyword arguments: {missing} for custom window function "
                         f"'{getattr(func, '__name__', func)}'.")
    return [kwargs[n] if n in kwargs else params[n].default for n in names]


def _window_values(func, kx, ky, kz, args, shape, dtype):
    """func on the broadcast grid kx x ky x kz: one call on arrays when the
    function is elementwise NumPy code, else one call per point."""
    try:
        with np.errstate(all="ignore"):
            v = np.asarray(func(kx, ky, kz, *args))
        if v.dtype != object:
            return np.broadcast_to(v, shape)
    except Exception:  # scalar-only code (math.*, branches on the arguments)
        pass
    one = np.vectorize(lambda a, b, c: func(float(a), float(b), float(c), *args), otypes=[dtype])
    return one(*np.broadcast_arrays(kx, ky, kz))


_SIGNS = ((1, 1, 1), (-1, 1, 1), (1, -1, 1), (1, 1, -1), (-1, -1, 1), (-1, 1, -1), (1, -1, -1), (-1, -1, -1))


def custom_window_kernel(func, args, L, bandwidth, power, mode, rows=8):
    """rFFT-grid kernel [L, L, L/2+1] of a user window W(kx, ky, kz, *args)
    (k in cycles per cell), built on the host in float64 like the reference:

    * ``full_rfft`` / ``complex_rfft`` (utils/convolution.py:74-252): for
      each image (ii, jj, kk) < bandwidth, eight terms P P P W at
      +(n L + x)/L and -(n L + L - x)/L per axis, summed in the reference's
      order; complex accumulation for ``complex_rfft``;
    * ``octant`` (:14-38, :264-283): W at (n L + i)/L for i in [0, L] on
      every axis, folded over the eight reflections i -> L - i.

    ``power`` holds |phi_hat(n/L)|^2 for n = 0..L*bandwidth."""
    P = np.asarray(power, dtype=np.float64)
    inv = 1.0 / L
    H = L // 2 + 1
    cplx = mode == "complex_rfft"
    dt = np.complex128 if cplx else np.float64
    y, z = np.arange(L), np.arange(H)
    if mode == "octant":
        n = np.arange(L + 1)
        arr = np.zeros((L + 1, L + 1, L + 1))
        for x0 in range(0, L + 1, rows):
            xs = n[x0:x0 + rows]
            acc = np.zeros((xs.size, L + 1, L + 1))
            for ii in range(bandwidth):
                ix = ii * L + xs
                for jj in range(bandwidth):
                    iy = jj * L + n
                    for kk in range(bandwidth):
                        iz = kk * L + n
                        w = _window_values(func, (ix * inv)[:, None, None], (iy * inv)[None, :, None],
                                           (iz * inv)[None, None, :], args, acc.shape, np.float64)
                        acc += P[ix][:, None, None] * P[iy][None, :, None] * P[iz][None, None, :] * w
            arr[x0:x0 + xs.size] = acc
        X, Xm = np.arange(L), L - np.arange(L)
        Y, Ym, Z, Zm = y, L - y, z, L - z
        # the reference's left-to-right sum of the eight reflections, one
        # gathered term at a time
        out = arr[np.ix_(X, Y, Z)]
        for ix, iy, iz in ((Xm, Y, Z), (X, Ym, Z), (X, Y, Zm), (Xm, Ym, Z), (Xm, Y, Zm), (X, Ym, Zm), (Xm, Ym, Zm)):
            out += arr[np.ix_(ix, iy, iz)]
        return out
    if mode not in ("full_rfft", "complex_rfft"):
        raise ValueError(f"Custom window functions do not support kernel_mode='{mode}'. "
                         "Use a real or complex RFFT kernel mode.")
    out = np.zeros((L, L, H), dtype=dt)
    for x0 in range(0, L, rows):
        xs = np.arange(x0, min(x0 + rows, L))
        acc = np.zeros((xs.size, L, H), dtype=dt)
        for ii in range(bandwidth):
            xi = (ii * L + xs, ii * L + L - xs)
            for jj in range(bandwidth):
                yi = (jj * L + y, jj * L + L - y)
                for kk in range(bandwidth):
                    zi = (kk * L + z, kk * L + L - z)
                    for sx, sy, sz in _SIGNS:
                        a, b, c = xi[sx < 0], yi[sy < 0], zi[sz < 0]
                        w = _window_values(func, (sx * a * inv)[:, None, None], (sy * b * inv)[None, :, None],
                                           (sz * c * inv)[None, None, :], args, acc.shape, dt)
                        acc += P[a][:, None, None] * P[b][None, :, None] * P[c][None, None, :] * w
        out[x0:x0 + xs.size] = acc
    return out


_POWER_CACHE = {}


def phi_power_device(phi_array, L, bandwidth, phi_resolution, device):
    """|phi_hat|^2 at n/L, n = 0..L*bw, as a float64 device tensor (cached)."""
    key = (id(phi_array), phi_array.shape[0], L, bandwidth, phi_resolution, str(device))
    hit = _POWER_CACHE.get(key)
    if hit is not None and hit[0] is phi_array:
        return hit[1]
    p = fourier_power_spectrum(phi_array, bandwidth, L * bandwidth, phi_resolution)
    t = torch.as_tensor(p, dtype=torch.float64, device=device)
    _POWER_CACHE[key] = (phi_array, t)
    return t


class WindowFunc(SFCField):
    is_window = True

    def __init__(self, win_params, sfc_params, bandwidth=1, threads=1, phi_array=None,
                 phi_fourier_power=None, device=None):
        super().__init__(threads=threads, device=device)
        missing = [k for k in self._REQUIRED_ARGV if k not in sfc_params]
        if missing:
            raise ValueError(f"WindowFunc missing required keys: {missing}")
        self.L = 1 << int(sfc_params["J"])
        self.J = int(sfc_params["J"])
        self.bandwidth = int(bandwidth)
        self.box_size = sfc_params["box_size"]
        self.phi_resolution = int(sfc_params["phi_resolution"])
        self.wavelet_mode = sfc_params["wavelet_mode"]
        self.wavelet_level = sfc_params["wavelet_level"]
        if self.L <= 0 or self.bandwidth <= 0:
            raise ValueError(f"Invalid L/bandwidth: L={self.L}, bandwidth={self.bandwidth}.")
        self.input_params = {**dict(win_params), "J": self.J, "box_size": self.box_size,
                             "phi_resolution": self.phi_resolution, "wavelet_mode": self.wavelet_mode,
                             "wavelet_level": self.wavelet_level, "bandwidth": self.bandwidth}
        if phi_array is None:
            phi_array = sfc_params.get("phi_array")
        if phi_array is None:
            phi_array = sample_scaling_function(self.wavelet_mode, self.wavelet_level)
        self.phi_array = np.asarray(phi_array, dtype=np.float64)
        self.phi_fourier_power = phi_fourier_power
        self.window_params = dict(win_params)
        # an explicit callable wins over a built-in type (io/window.py:88-96)
        custom = win_params.get("func")
        self.has_custom_func = custom is not None
        if self.has_custom_func:
            if not callable(custom):
                raise TypeError("Custom window parameter 'func' must be callable.")
            self.type = win_params.get("type") or "custom"
            self.func = custom
        elif win_params.get("type") in COMPLEX_FULL_FFT_WINDOW_TYPES:
            self.type = win_params["type"]
            self.func = None
        else:
            if "type" not in win_params or win_params["type"] not in WIN_CODES:
                raise ValueError(f"Unsupported input window function type: {win_params.get('type')}. "
                                 f"Supported types: {', '.join(WIN_CODES)}")
            self.type = win_params["type"]
            self.func = None
        km = win_params.get("kernel_mode") or default_kernel_mode(self.type, self.has_custom_func)
        self.kernel_mode = normalize_kernel_mode(km)
        self.input_params["kernel_mode"] = self.kernel_mode
        self.window_params["kernel_mode"] = self.kernel_mode
        self.len_args = plain_copy(win_params.get("len_args", {})) or {}
        self.input_params["len_args"] = plain_copy(self.len_args)
        self.window_params["len_args"] = plain_copy(self.len_args)
        self.rescale_len_args = {k: v * self.L / self.box_size for k, v in self.len_args.items()
                                 if v is not None}
        self.los_args = normalize_los_args(win_params.get("los_args", {}),
                                           None if self.has_custom_func else self.type)
        self.other_args = win_params.get("other_args", {}) or {}
        self.input_params["los_args"] = self.los_args
        self.window_params["los_args"] = self.los_args
        self.window_args = dict(self.rescale_len_args)
        self.window_args.update(self.los_args)
        self.window_args.update(plain_copy(self.other_args))
        if self.type == "thick_shell" and not self.has_custom_func:
            try:
                r = float(self.rescale_len_args["R"])
                d = float(self.rescale_len_args["delta_R"])
            except (KeyError, TypeError, ValueError) as exc:
                raise ValueError("thick_shell requires finite len_args {'R': ..., 'delta_R': ...}.") from exc
            if not np.isfinite(r) or r < 0.0:
                raise ValueError("thick_shell requires a finite non-negative R.")
            if not np.isfinite(d) or d <= 0.0:
                raise ValueError("thick_shell requires a finite positive delta_R.")
        self.w_kernel = None
        self._kernel_dev = None
        self.is_composite_window = False
        self._scale = 1.0

    # ---- mode resolution (io/window.py:150-195) ---------------------------
    def _los_is_axis_aligned(self):
        has_complete = all(k in self.los_args for k in LOS_ARG_KEYS)
        if self.has_custom_func:
            if not has_complete:
                return False
        elif self.type not in ANISOTROPIC_AUTO_WINDOW_TYPES and not has_complete:
            return True
        los = np.array([float(self.los_args.get("nx", 0.0)), float(self.los_args.get("ny", 0.0)),
                        float(self.los_args.get("nz", 1.0))])
        n = np.linalg.norm(los)
        if n == 0.0:
            return True
        los = np.abs(los / n)
        return bool(any(np.isclose(los[i], 1.0) and np.isclose(los[(i + 1) % 3], 0.0)
                        and np.isclose(los[(i + 2) % 3], 0.0) for i in range(3)))

    def resolved_mode(self):
        """The kernel builder the reference would use: octant / full_rfft /
        complex_rfft / complex_full_fft (io/window.py:274-332)."""
        t, m = self.type, self.kernel_mode
        if self.has_custom_func:
            if m == "complex_full_fft":
                raise ValueError("Custom window functions do not support kernel_mode='complex_full_fft'. "
                                 "Use a real or complex RFFT kernel mode.")
            if m in ("octant", "full_rfft", "complex_rfft"):
                return m
            return "octant" if self._los_is_axis_aligned() else "full_rfft"
        if t in COMPLEX_RFFT_WINDOW_TYPES and m == "octant":
            raise ValueError(f"Window type '{t}' is complex and directional; use kernel_mode='complex_rfft' or 'auto'.")
        if t in COMPLEX_FULL_FFT_WINDOW_TYPES and m not in ("auto", "complex_full_fft"):
            raise ValueError(f"Window type '{t}' requires kernel_mode='complex_full_fft' or 'auto'.")
        if m == "complex_full_fft" or (m == "auto" and t in COMPLEX_FULL_FFT_WINDOW_TYPES):
            return "complex_full_fft"
        if m == "complex_rfft" or (m in ("auto", "full_rfft") and t in COMPLEX_RFFT_WINDOW_TYPES):
            return "complex_rfft"
        if m == "full_rfft":
            return "full_rfft"
        if m == "octant":
            return "octant"
        return "octant" if self._los_is_axis_aligned() else "full_rfft"

    # ---- device descriptor --------------------------------------------------
    @property
    def materialized(self):
        """True when the kernel is a stored array (composite, loaded or
        custom-function windows) rather than evaluated on the fly."""
        return self.is_composite_window or self.has_custom_func

    def descriptor(self):
        if self.has_custom_func:
            raise ValueError("A custom window function has no built-in descriptor; use its materialised kernel.")
        mode = self.resolved_mode()
        if mode == "complex_full_fft":
            raise ValueError("complex_full_fft windows are handled by the multipole engine.")
        d = HermesWindow()
        d.type = WIN_CODES[self.type]
        d.kernel_mode = KMODE[mode]
        d.zero_mode_zero = 1 if self.type in ZERO_MODE_ZERO_WINDOW_TYPES else 0
        names = WIN_ARGS[self.type]
        for i, nm in enumerate(names):
            if nm not in self.window_args or self.window_args[nm] is None:
                raise ValueError(f"Missing keyword arguments: ['{nm}'] for window '{self.type}'")
            d.len[i] = float(self.window_args[nm])
        los = self.los_args if self.los_args else DEFAULT_LOS_ARGS
        for i, k in enumerate(LOS_ARG_KEYS):
            d.los[i] = float(los.get(k, DEFAULT_LOS_ARGS[k]))
        d.scale = float(self._scale)
        return d

    def phi_power(self):
        if self.phi_fourier_power is not None:
            return torch.as_tensor(np.asarray(self.phi_fourier_power, dtype=np.float64), device=self.device)
        return phi_power_device(self.phi_array, self.L, self.bandwidth, self.phi_resolution, self.device)

    @property
    def is_complex(self):
        if self.is_composite_window:
            return self._kernel_dev.is_complex()
        if self.has_custom_func:
            return self.resolved_mode() == "complex_rfft"
        return self.resolved_mode() in ("complex_rfft", "complex_full_fft")

    def kernel_device(self):
        """Materialised rFFT-grid kernel as a device tensor (float32 or complex64)."""
        if self._kernel_dev is not None:
            return self._kernel_dev
        if self.has_custom_func:
            # io/window.py:274-332 with utils/convolution.py: built on the host
            # (a Python callable), kept on the device for the convolutions
            args = ordered_window_args(self.func, self.window_args)
            pw = self.phi_power().double().cpu().numpy()
            k = custom_window_kernel(self.func, args, self.L, self.bandwidth, pw, self.resolved_mode())
            self.w_kernel = k
            self._kernel_dev = torch.as_tensor(k.astype(np.complex64) if np.iscomplexobj(k)
                                               else k.astype(np.float32), device=self.device)
            return self._kernel_dev
        if self.resolved_mode() == "complex_full_fft":
            from .multipole import complex_full_kernel

            self._kernel_dev = complex_full_kernel(self)
            return self._kernel_dev
        L, H = self.L, self.L // 2 + 1
        d = self.descriptor()
        pw = self.phi_power()
        lib = _lib.load()
        if d.kernel_mode == KMODE["complex_rfft"]:
            k = torch.empty((L, L, H), dtype=torch.complex64, device=self.device)
            rc = lib.hermes_window_materialize(ctypes.byref(d), _ptr(pw), self.bandwidth, self.J, None,
                                               _ptr(k), _stream_ptr(self.device))
        else:
            k = torch.empty((L, L, H), dtype=torch.float32, device=self.device)
            rc = lib.hermes_window_materialize(ctypes.byref(d), _ptr(pw), self.bandwidth, self.J, _ptr(k),
                                               None, _stream_ptr(self.device))
        _lib.check(rc, "hermes_window_materialize")
        self._kernel_dev = k
        return k

    def as_array(self):
        if self.w_kernel is None:
            t = self.kernel_device()
            if self.w_kernel is None:  # custom windows keep their float64 host kernel
                self.w_kernel = (t.to(torch.complex128) if t.is_complex() else t.to(torch.float64)).cpu().numpy()
        return self.w_kernel

    def copy(self, copy_kernel=True):
        """A copy that does not rebuild the kernel (io/window.py:487-516):
        with copy_kernel the stored kernel (host and device) is copied, else
        the copy rebuilds it on its next use.  The window callable is shared."""
        if self.is_composite_window and not copy_kernel:
            raise ValueError("Composite WindowFunc cannot be copied with copy_kernel=False.")
        new = self.__class__.__new__(self.__class__)
        for key, value in self.__dict__.items():
            if key == "func":
                new.func = value
            elif key in ("w_kernel", "_kernel_dev"):
                keep = copy_kernel and value is not None
                setattr(new, key, (value.clone() if isinstance(value, torch.Tensor) else value.copy()) if keep
                        else None)
            elif isinstance(value, np.ndarray):
                setattr(new, key, value.copy())
            elif isinstance(value, torch.Tensor):
                setattr(new, key, value.clone())
            else:
                setattr(new, key, copy.deepcopy(value))
        return new

    # ---- persistence (io/window.py:518-548, io/base.py:24-121) ---------------
    def save(self, f_out, single=True, overwrite=False, **flags):
        """Framed pickle {**input_params, 'window_kernal': kernel} as the
        reference writes it (io/window.py:530-548; the key's spelling is
        the reference's), at the path check_fout resolves (returned)."""
        from .sfc_field import check_fout, write_numpy_pickle

        if any(flags.values()):
            raise ValueError("WindowFunc.save writes the window file only.")
        if not self.input_params:
            raise ValueError('The dict_argv "win_params" is empty.')
        f_out = check_fout(self, f_out, overwrite)
        if f_out:
            with open(f_out, "wb") as f:
                write_numpy_pickle(f, {**self.input_params, "window_kernal": self.as_array()})
        return f_out

    def load(self, f_in, single=True, **flags):
        """Reads a saved window: input_params from the file and its kernel,
        used from then on as a materialised kernel."""
        from .sfc_field import read_numpy_pickle

        with open(f_in, "rb") as f:
            dataset = read_numpy_pickle(f)
        if "window_kernal" not in dataset:
            raise ValueError("Failed to load the dataset. The file is missing the 'window_kernal' key.")
        self.input_params = {k: v for k, v in dataset.items() if k != "window_kernal"}
        k = np.asarray(dataset["window_kernal"])
        self.w_kernel = k
        self._kernel_dev = torch.as_tensor(k.astype(np.complex64) if np.iscomplexobj(k) else k.astype(np.float32),
                                           device=self.device)
        self.is_composite_window = True

    # ---- composite algebra (io/window.py:364-485) ----------------------------
    def _spawn_composite(self, kernel, operation):
        new = self.__class__.__new__(self.__class__)
        new.__dict__.update({k: copy.copy(v) for k, v in self.__dict__.items()})
        new.type = "composite"
        new.has_custom_func, new.func = False, None
        new.kernel_mode = "materialized"
        new.len_args, new.rescale_len_args, new.los_args, new.window_args = {}, {}, {}, {}
        new.other_args = {"operation": copy.deepcopy(operation)}
        new.window_params = {"type": new.type, "len_args": {}, "los_args": {}, "other_args": new.other_args,
                             "kernel_mode": new.kernel_mode}
        new.input_params = {**copy.deepcopy(new.window_params), "J": self.J, "box_size": self.box_size,
                            "phi_resolution": self.phi_resolution, "wavelet_mode": self.wavelet_mode,
                            "wavelet_level": self.wavelet_level, "bandwidth": self.bandwidth}
        new.w_kernel = None
        new._kernel_dev = kernel
        new.is_composite_window = True
        return new

    def _check_compat(self, other):
        for key in ("L", "bandwidth", "box_size", "phi_resolution", "wavelet_mode", "wavelet_level"):
            if getattr(self, key) != getattr(other, key):
                raise ValueError(f"Cannot combine WindowFunc objects with different {key}.")

    def _binop(self, other, name, fn):
        if not isinstance(other, WindowFunc):
            return NotImplemented
        self._check_compat(other)
        a, b = self.kernel_device(), other.kernel_device()
        return self._spawn_composite(fn(a, b), {"op": name, "left": self.window_params,
                                                "right": other.window_params})

    def _scalar(self, s, name, fn):
        if not (np.isscalar(s) and not isinstance(s, (str, bytes)) and np.isrealobj(s)):
            return NotImplemented
        return self._spawn_composite(fn(self.kernel_device(), float(s)),
                                     {"op": name, "window": self.window_params, "scalar": float(s)})

    def __add__(self, other):
        return self._binop(other, "add", lambda a, b: a + b)

    def __sub__(self, other):
        return self._binop(other, "sub", lambda a, b: a - b)

    def __neg__(self):
        return self._scalar(-1.0, "mul", lambda a, s: a * s)

    def __mul__(self, other):
        if isinstance(other, WindowFunc):
            return self._binop(other, "projected_kernel_product", lambda a, b: a * b)
        return self._scalar(other, "mul", lambda a, s: a * s)

    def __rmul__(self, other):
        return self.__mul__(other)

    def __truediv__(self, other):
        if np.isscalar(other) and float(other) == 0.0:
            raise ZeroDivisionError("Cannot divide WindowFunc by zero.")
        return self._scalar(other, "div", lambda a, s: a / s)


_WS = {}


def _workspace(key, nbytes, device):
    buf = _WS.get((key, str(device)))
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
        _WS[(key, str(device))] = buf
    return buf


def apply_window(eps, window, out=None):
    """Real field (float32 [L,L,L] device tensor) convolved with a window."""
    lib = _lib.load()
    J = window.J
    if out is None:
        out = torch.empty_like(eps)
    dev = eps.device
    sptr = _stream_ptr(dev)
    need = ctypes.c_size_t(0)
    _lib.check(lib.hermes_window_workspace_size(J, ctypes.byref(need)), "window_workspace_size")
    ws = _workspace("spectrum", need.value, dev)
    if window.materialized:
        k = window.kernel_device()
        _lib.check(lib.hermes_fft_r2c(_ptr(eps), _ptr(ws), J, sptr), "hermes_fft_r2c")
        kr = k if not k.is_complex() else None
        kc = k if k.is_complex() else None
        _lib.check(lib.hermes_spectrum_multiply(_ptr(ws), _ptr(kr), _ptr(kc), J, 1.0 / float(window.L) ** 3,
                                                sptr), "hermes_spectrum_multiply")
        _lib.check(lib.hermes_fft_c2r(_ptr(ws), _ptr(out), J, sptr), "hermes_fft_c2r")
        return out
    d = window.descriptor()
    pw = window.phi_power()
    _lib.check(lib.hermes_window_apply(_ptr(eps), _ptr(out), J, ctypes.byref(d), _ptr(pw), window.bandwidth,
                                       _ptr(ws), ws.numel(), sptr), "hermes_window_apply")
    return out


def convolve_field(field, window):
    """SFCField @ WindowFunc (io/sfc_field.py:93-150) on the GPU."""
    if not isinstance(window, WindowFunc):
        raise TypeError(f"Convolution requires a WindowFunc on the right-hand side; got {type(window)}.")
    eps = field.epsilon_device
    if eps is None or eps.ndim != 3:
        raise ValueError("Convolution expects a 3D field.")
    if eps.shape[0] != window.L:
        raise ValueError(f"Convolution requires same shape; field L={eps.shape[0]}, window L={window.L}.")
    mode = "materialized" if window.materialized else window.resolved_mode()
    if mode == "complex_full_fft":
        from .multipole import convolve_complex_full

        out = convolve_complex_full(field, window)
    elif mode == "materialized" and window.kernel_device().shape[-1] == window.L:
        # a stored complex full-FFT kernel (a composite of legendre /
        # radial multipole windows): ifftn(fftn(eps) K), io/sfc_field.py:118-121
        k = window.kernel_device()
        out = torch.fft.ifftn(torch.fft.fftn(eps.to(torch.complex64)) * k.to(torch.complex64))
    else:
        out = apply_window(eps.to(torch.float32).contiguous(), window)
    new = field._spawn_like()
    new._eps_dev = out
    windows = field.sfc_info.get("convolution_of", [])
    new.sfc_info.update({"convolution_of": windows + [window.window_params]})
    field._mark_derived(new)
    new.format_sfc_params()
    return new


def rfft_field(eps):
    """Half spectrum (complex64 [L,L,L/2+1]) of a float32 field."""
    L = eps.shape[0]
    J = L.bit_length() - 1
    spec = torch.empty((L, L, L // 2 + 1), dtype=torch.complex64, device=eps.device)
    _lib.check(_lib.load().hermes_fft_r2c(_ptr(eps), _ptr(spec), J, _stream_ptr(eps.device)), "hermes_fft_r2c")
    return spec


def materialized_pair_products(fields, pairs, windows, exclude_k0=True):
    """pair_products for windows with a stored kernel (custom callables,
    composites): mean over cells of (f_i convolved with K) * f_j, the
    reference's own form of the product (theory/corr2pcf.py:366-382), with
    the convolution on hermes_fft_r2c / hermes_spectrum_multiply /
    hermes_fft_c2r and the cell sum in float64.  fields: float32 [L,L,L]
    device tensors.  Same return as pair_products."""
    n_bins, n_pairs = len(windows), len(pairs)
    out = np.zeros((n_bins, n_pairs), dtype=np.float64)
    k0 = np.zeros(n_bins, dtype=np.float64)
    dcs = [float(f.double().sum().item()) for f in fields]
    # mean-free copies carry every k != 0 mode: the k = 0 term is added in
    # float64 below instead of surviving a float32 cancellation
    cen = [(f.double() - dc / f.numel()).to(torch.float32).contiguous() for f, dc in zip(fields, dcs)]
    for b, w in enumerate(windows):
        if not w.materialized:
            raise ValueError("materialized_pair_products takes windows with a stored kernel.")
        L3 = float(w.L) ** 3
        k0[b] = float(w.kernel_device()[0, 0, 0].real.item())
        convs = {}
        for c, (i, j) in enumerate(pairs):
            if i not in convs:
                convs[i] = apply_window(cen[i], w)
            v = float((convs[i].double() * cen[j].double()).sum().item()) / L3
            out[b, c] = v + (0.0 if exclude_k0 else k0[b] * dcs[i] * dcs[j] / L3 ** 2)
    return out, k0


def family_descriptors(template, len_args_list):
    """Descriptors of a family of built-in windows that differ from
    `template` only in their physical len_args (one dict per member): the
    template's descriptor with each member's lengths rescaled to grid units,
    as WindowFunc.descriptor() gives for the member itself."""
    base = template.descriptor()
    names = WIN_ARGS[template.type]
    L, box = template.L, template.box_size
    arr = (HermesWindow * len(len_args_list))()
    size = ctypes.sizeof(HermesWindow)
    for i, la in enumerate(len_args_list):
        ctypes.memmove(ctypes.byref(arr[i]), ctypes.byref(base), size)
        for j, nm in enumerate(names):
            v = la.get(nm)
            if v is None:
                raise ValueError(f"Missing keyword arguments: ['{nm}'] for window '{template.type}'")
            arr[i].len[j] = float(v * L / box)  # the rescale order of WindowFunc.__init__
        if template.type == "thick_shell" and not (arr[i].len[0] >= 0.0 and arr[i].len[1] > 0.0
                                                   and np.isfinite(arr[i].len[0]) and np.isfinite(arr[i].len[1])):
            raise ValueError("thick_shell requires a finite non-negative R and a finite positive delta_R.")
    return arr


def pair_products(spectra, pairs, windows, exclude_k0=True, descs=None):
    """sum_k F_i K_b conj(F_j) / L^6 for every window b and pair (i, j).

    spectra: list of complex64 half spectra; pairs: list of (i, j);
    windows: list of WindowFunc (built-in, non-composite), or the template of
    a family whose descriptors are given in `descs` (family_descriptors).
    Returns a float64 array [n_bins, n_pairs] and the kernel values at
    k = 0 [n_bins].
    """
    lib = _lib.load()
    w0 = windows[0]
    J, dev = w0.J, spectra[0].device
    n_pairs = len(pairs)
    if descs is None:
        descs = (HermesWindow * len(windows))(*[w.descriptor() for w in windows])
    n_bins = len(descs)
    ptrs = (ctypes.c_void_p * len(spectra))(*[s.data_ptr() for s in spectra])
    pr = (ctypes.c_int32 * (2 * n_pairs))(*[v for p in pairs for v in p])
    need = ctypes.c_size_t(0)
    _lib.check(lib.hermes_pair_products_workspace_size(J, n_bins, n_pairs, ctypes.byref(need)),
               "pair_products_workspace_size")
    ws = _workspace("pair_products", need.value, dev)
    out = np.zeros(n_bins * n_pairs, dtype=np.float64)
    k0 = np.zeros(n_bins, dtype=np.float64)
    pw = w0.phi_power()
    rc = lib.hermes_pair_products(ptrs, len(spectra), pr, n_pairs, descs, n_bins, _ptr(pw), w0.bandwidth, J,
                                  1 if exclude_k0 else 0, out.ctypes.data_as(ctypes.c_void_p),
                                  k0.ctypes.data_as(ctypes.c_void_p), _ptr(ws), ws.numel(), _stream_ptr(dev))
    _lib.check(rc, "hermes_pair_products")
    return out.reshape(n_bins, n_pairs), k0
