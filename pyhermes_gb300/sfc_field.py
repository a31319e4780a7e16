"""``SFCField``: a scaling-function-coefficient field resident in GB300 HBM.

Mirrors the reference container ``pyhermes/io/sfc_field.py:50-584``:
``sfc_info`` metadata (every key is also an attribute), ``epsilon``,
``field @ window`` convolution, + - * / algebra, weight-normalisation
switches, ``field_mean_density`` and NumPy-framed pickle save/load.

Differences by design: the coefficients live on the GPU as a float32 torch
tensor (``epsilon_device``); ``epsilon`` returns a float64 NumPy copy made
on first access (the reference's dtype), so reference tools that read
``.epsilon`` keep working.  Arithmetic stays on the device.
"""

import copy
import logging
import math
import os
import pickle
from io import BytesIO

import numpy as np
import torch

logger = logging.getLogger(__name__)

REQUIRED_ARGV = ("J", "box_size", "phi_resolution", "wavelet_mode", "wavelet_level")


def normalize_weight_normalization(weight_normalization):
    """pyhermes/io/sfc_field.py:21-29."""
    if weight_normalization is None:
        raise ValueError("weight_normalization must be one of 'raw', 'catalog', 'field', or 'unit'.")
    mode = str(weight_normalization).strip().lower()
    if mode == "unit":
        return "field"
    if mode not in {"raw", "catalog", "field"}:
        raise ValueError("weight_normalization must be one of 'raw', 'catalog', 'field', or 'unit'.")
    return mode


def normalize_task_weight_normalization(weight_normalization):
    """pyhermes/io/sfc_field.py:32-38."""
    if weight_normalization is None:
        raise ValueError("task weight_normalization must be one of 'raw', 'catalog', 'field', or 'unit'.")
    mode = str(weight_normalization).strip().lower()
    if mode not in {"raw", "catalog", "field", "unit"}:
        raise ValueError("task weight_normalization must be one of 'raw', 'catalog', 'field', or 'unit'.")
    return mode


def normalize_field_value_normalization(normalization):
    """pyhermes/io/sfc_field.py:41-47."""
    if normalization is None:
        return None
    mode = str(normalization).strip().lower()
    if mode not in {"raw", "catalog", "field", "unit"}:
        raise ValueError("normalization must be None, 'raw', 'catalog', 'field', or 'unit'.")
    return mode


def check_fout(instance, fout_path, overwrite=False):
    """Output path rules of the reference's savers (io/funcs.py:13-57):
    no path -> None (nothing written); an existing file is replaced only
    with overwrite, else the first free ``name_<n>.ext`` is used; a folder
    (existing, or a path ending in a separator) receives
    ``Output_<Class>_<YYYYmmddHHMM>.pkl``; missing parent folders are made."""
    import datetime

    if fout_path is None or fout_path == "":
        logger.info("No <fout_path> specified, skipping disk output.")
        return None
    fout_path = os.fspath(fout_path)
    is_folder = fout_path.endswith(("/", "\\"))
    if os.path.exists(fout_path):
        if os.path.isdir(fout_path):
            is_folder = True
        elif os.path.isfile(fout_path):
            if overwrite:
                logger.warning("Output file '%s' already exists and will be overwritten (overwrite=True).",
                               fout_path)
            else:
                logger.warning("Output file '%s' already exists! Generating a new file name.", fout_path)
                base, ext = os.path.splitext(fout_path)
                n = 1
                while os.path.exists(f"{base}_{n}{ext}"):
                    n += 1
                fout_path = f"{base}_{n}{ext}"
    if not is_folder:
        parent = os.path.dirname(fout_path)
        if parent:
            os.makedirs(parent, exist_ok=True)
        return fout_path
    os.makedirs(fout_path, exist_ok=True)
    stamp = datetime.datetime.now().strftime("%Y%m%d%H%M")
    return os.path.join(fout_path, f"Output_{instance.__class__.__name__}_{stamp}.pkl")


def write_numpy_pickle(file_obj, value, protocol=4):
    """NumPy-framed pickle (pyhermes/io/pickle_compat.py:87-90): the pickle
    bytes stored as a uint8 .npy array."""
    payload = pickle.dumps(_normalize_pathlike(value), protocol=protocol)
    np.lib.format.write_array(file_obj, np.frombuffer(payload, dtype=np.uint8))


def read_numpy_pickle(file_obj):
    """pyhermes/io/pickle_compat.py:81-84."""
    serialized = np.lib.format.read_array(file_obj, allow_pickle=False)
    return pickle.load(BytesIO(serialized.tobytes()))


def _normalize_pathlike(value):
    if isinstance(value, os.PathLike):
        return os.fsdecode(os.fspath(value))
    if isinstance(value, dict):
        return {_normalize_pathlike(k): _normalize_pathlike(v) for k, v in value.items()}
    if isinstance(value, list):
        return [_normalize_pathlike(v) for v in value]
    if isinstance(value, tuple):
        return tuple(_normalize_pathlike(v) for v in value)
    return value


_SAVE_FLAGS = (("save_sfc_field", "save_sfc_field"), ("save_counting", "save_counting"),
               ("save_2pcf", "save_corr2pcf"), ("save_3pcf", "save_corr3pcf"),
               ("save_3pcf_multipole", "save_corr3pcf_multipole"))
_READ_FLAGS = (("read_sfc_field", "load_sfc_field"), ("read_counting", "load_counting"),
               ("read_2pcf", "load_corr2pcf"), ("read_3pcf", "load_corr3pcf"),
               ("read_3pcf_multipole", "load_corr3pcf_multipole"))


class ResultFileIO:
    """The generic ``save`` / ``load`` of the reference's data containers
    (io/base.py:24-124): a flag names the file kind, which must be the
    container's own; without a flag the container's own kind is used."""

    _OWN_SAVE = ""
    _OWN_LOAD = ""

    def save(self, f_out, save_sfc_field=False, save_counting=False, save_2pcf=False, save_3pcf=False,
             save_3pcf_multipole=False, single=True, overwrite=False):
        flags = dict(zip((k for k, _ in _SAVE_FLAGS),
                         (save_sfc_field, save_counting, save_2pcf, save_3pcf, save_3pcf_multipole)))
        picked = [m for k, m in _SAVE_FLAGS if flags[k]] or [self._OWN_SAVE]
        if picked != [self._OWN_SAVE]:
            raise ValueError(f"{type(self).__name__} cannot be saved as {picked[0].split('_', 1)[1]}.")
        return getattr(self, self._OWN_SAVE)(f_out, overwrite=overwrite)

    def load(self, f_in, read_sfc_field=False, read_counting=False, read_2pcf=False, read_3pcf=False,
             read_3pcf_multipole=False, single=True):
        flags = dict(zip((k for k, _ in _READ_FLAGS),
                         (read_sfc_field, read_counting, read_2pcf, read_3pcf, read_3pcf_multipole)))
        picked = [m for k, m in _READ_FLAGS if flags[k]] or [self._OWN_LOAD]
        if picked != [self._OWN_LOAD]:
            raise ValueError(f"{type(self).__name__} cannot read a {picked[0].split('_', 1)[1]} file.")
        getattr(self, self._OWN_LOAD)(f_in)


def describe_input(value):
    """A task input as the reference records it in result files
    (theory/corr2pcf.py:174-208): strings and 'uniform' as given, numbers as
    float, a field or window object as a short summary, dicts copied."""
    if value is None or isinstance(value, str):
        return value
    if isinstance(value, (float, int, np.floating)):
        return float(value)
    from .params import serialize_window_params

    if getattr(value, "is_window", False):
        return {"kind": "WindowFunc", "type": getattr(value, "type", "custom"),
                "len_args": serialize_window_params(getattr(value, "len_args", {}) or {}),
                "los_args": serialize_window_params(getattr(value, "los_args", {}) or {}),
                "other_args": serialize_window_params(getattr(value, "other_args", {}) or {})}
    if isinstance(value, SFCField):
        return {"kind": "SFCField", "L": value.L, "box_size": value.box_size, "wavelet_mode": value.wavelet_mode,
                "wavelet_level": value.wavelet_level}
    if isinstance(value, dict):
        # window dicts as utils/window_params.py:104-121 serialises them
        return serialize_window_params(value)
    return value


class SFCField:
    _REQUIRED_ARGV = REQUIRED_ARGV

    def __init__(self, *args, threads=None, data_path=None, device=None, **kwargs):
        self.threads = threads
        self.sfc_info = {}
        self.task_params = {}
        self.saveflag = False
        self.device = torch.device(device) if device is not None else torch.device("cuda")
        self._eps_dev = None
        self._eps_host = None
        if data_path:
            self.sfc_info["sfc_field_path"] = data_path
            self.load_sfc_field(data_path)

    # ---- coefficient storage -------------------------------------------
    @property
    def epsilon_device(self):
        if self._eps_dev is None and self._eps_host is not None:
            self._eps_dev = torch.as_tensor(self._eps_host, device=self.device).to(
                torch.float32 if not np.iscomplexobj(self._eps_host) else torch.complex64)
        return self._eps_dev

    @epsilon_device.setter
    def epsilon_device(self, t):
        self._eps_dev = t
        self._eps_host = None

    @property
    def epsilon(self):
        if self._eps_host is None and self._eps_dev is not None:
            t = self._eps_dev
            t = t.to(torch.complex128) if t.is_complex() else t.to(torch.float64)
            self._eps_host = t.cpu().numpy()
        return self._eps_host

    @epsilon.setter
    def epsilon(self, value):
        if value is None:
            self._eps_dev = None
            self._eps_host = None
        elif isinstance(value, torch.Tensor):
            self.epsilon_device = value
        else:
            self._eps_host = np.asarray(value)
            self._eps_dev = None

    def as_array(self):
        return self.epsilon

    # ---- metadata ----------------------------------------------------------
    def format_sfc_params(self):
        missing = [k for k in self._REQUIRED_ARGV if k not in self.sfc_info]
        if missing:
            raise ValueError(f"SFCField missing required keys: {missing}")
        for key, value in self.sfc_info.items():
            setattr(self, key, value)

    def _spawn_like(self):
        new = self.__class__.__new__(self.__class__)
        new.threads = self.threads
        new.sfc_info = copy.deepcopy(self.sfc_info)
        new.task_params = copy.deepcopy(getattr(self, "task_params", {}))
        new.saveflag = False
        new.device = self.device
        new._eps_dev = None
        new._eps_host = None
        return new

    def copy(self):
        new = self._spawn_like()
        if self._eps_dev is not None:
            new._eps_dev = self._eps_dev.clone()
        elif self._eps_host is not None:
            new._eps_host = self._eps_host.copy()
        new.format_sfc_params()
        return new

    def _derived_field_integral(self, field):
        t = field.epsilon_device
        if t is None:
            return None
        total = t.to(torch.complex128 if t.is_complex() else torch.float64).sum().item()
        if isinstance(total, complex):
            if not (np.isfinite(total.real) and np.isfinite(total.imag)):
                return None
            if abs(total.imag) <= 1e-12 * max(1.0, abs(total.real)):
                return float(total.real)
            return complex(total)
        return float(total) if np.isfinite(total) else None

    def _mark_derived(self, field):
        """pyhermes/io/sfc_field.py:326-338."""
        field.sfc_info.update({
            "catalog_weight_sum": None,
            "catalog_weight_sq_sum": None,
            "raw_field_weighted_sum": None,
            "field_integral": self._derived_field_integral(field),
            "weight_normalization": None,
            "particle_count": None,
            "particle_data_retrievable": False,
            "particle_data_path": "",
            "particle_data_format": "",
            "field_kind": "derived_field",
        })

    # ---- algebra (device) ----------------------------------------------------
    def _binary(self, other, op):
        if isinstance(other, SFCField):
            a, b = self.epsilon_device, other.epsilon_device
            if a is None or b is None:
                raise ValueError("Cannot operate on a field whose epsilon is None.")
            if a.shape != b.shape:
                raise ValueError(f"Shape mismatch: {tuple(a.shape)} vs {tuple(b.shape)}")
            res = op(a, b)
        elif np.isscalar(other) and not isinstance(other, (str, bytes)):
            if self.epsilon_device is None:
                raise ValueError("Cannot operate on a field whose epsilon is None.")
            res = op(self.epsilon_device, other)
        else:
            return NotImplemented
        new = self._spawn_like()
        new._eps_dev = res
        self._mark_derived(new)
        new.format_sfc_params()
        return new

    def __add__(self, other):
        return self._binary(other, lambda a, b: a + b)

    def __radd__(self, other):
        return self._binary(other, lambda a, b: b + a)

    def __sub__(self, other):
        return self._binary(other, lambda a, b: a - b)

    def __rsub__(self, other):
        return self._binary(other, lambda a, b: b - a)

    def __mul__(self, other):
        return self._binary(other, lambda a, b: a * b)

    def __rmul__(self, other):
        return self._binary(other, lambda a, b: b * a)

    def __truediv__(self, other):
        if np.isscalar(other) and float(other) == 0.0:
            raise ZeroDivisionError("Cannot divide SFCField by zero.")
        if isinstance(other, SFCField):
            return NotImplemented
        return self._binary(other, lambda a, b: a / b)

    def __matmul__(self, other):
        from .window import convolve_field

        if hasattr(other, "as_array") and not isinstance(other, SFCField) or getattr(other, "is_window", False):
            return convolve_field(self, other)
        return NotImplemented

    def __rmatmul__(self, other):
        """io/sfc_field.py:157-160: field @ window reached from the window's side."""
        from .window import convolve_field

        if isinstance(other, SFCField) and getattr(self, "is_window", False):
            return convolve_field(other, self)
        return NotImplemented

    # ---- normalisation -----------------------------------------------------
    def _normalization_denominator(self, weight_normalization):
        """pyhermes/io/sfc_field.py:340-352."""
        mode = normalize_weight_normalization(weight_normalization)
        if mode == "raw":
            return 1.0
        if mode == "catalog":
            value, label = getattr(self, "catalog_weight_sum", None), "catalog_weight_sum"
        else:
            value, label = getattr(self, "raw_field_weighted_sum", None), "raw_field_weighted_sum"
        if value is None or not np.isfinite(value) or np.isclose(value, 0.0):
            raise ValueError(f"Cannot use weight_normalization='{mode}' without a finite, non-zero {label}.")
        return float(value)

    def _field_integral_for_normalization(self, weight_normalization):
        raw_sum = getattr(self, "raw_field_weighted_sum", None)
        if raw_sum is None or not np.isfinite(raw_sum):
            return None
        return float(raw_sum / self._normalization_denominator(weight_normalization))

    def get_particle_data(self):
        """pyhermes/io/sfc_field.py:425-482: the catalogue behind a catalog
        field -- from the saved particle dataset (particle_data_path) or by
        re-reading fin -- with catalogue weights, normalised weights, field
        values and the projection weights of the field's normalisation."""
        if getattr(self, "field_kind", None) != "catalog_field":
            raise ValueError("Only catalog fields can provide particle data. Derived fields do not retain a unique "
                             "particle catalogue.")
        if not bool(getattr(self, "particle_data_retrievable", True)):
            raise ValueError("This field no longer maps to one retrievable particle catalogue. Provide particle_pos1 "
                             "and particle_weight1 explicitly for particle-centred statistics.")
        den = self._normalization_denominator(getattr(self, "weight_normalization", "raw"))
        path = self.sfc_info.get("particle_data_path", "")
        if path:
            with np.load(path) as z:
                if not {"pos", "catalog_weight", "field_value"}.issubset(z.files):
                    raise ValueError(f"Particle dataset '{path}' must contain ['catalog_weight', 'field_value', 'pos'] "
                                     "arrays.")
                pos = z["pos"]
                cw = np.asarray(z["catalog_weight"], dtype=np.float64)
                fv = np.asarray(z["field_value"], dtype=np.float64)
        else:
            raise ValueError("This field has no saved particle dataset (save_particle_data); catalogue files are "
                             "read by the caller, so pass the particle positions and weights explicitly.")
        return {"pos": pos, "catalog_weight": cw, "normalized_catalog_weight": cw / float(self.catalog_weight_sum),
                "field_value": fv, "projection_weight": cw * fv / den}

    def switch_weight_normalization(self, weight_normalization):
        """pyhermes/io/sfc_field.py:360-378 (rescale by old_den/new_den)."""
        mode = normalize_weight_normalization(weight_normalization)
        if getattr(self, "field_kind", None) != "catalog_field":
            raise ValueError("weight normalization can only be switched for catalog fields.")
        new = self.copy()
        current = normalize_weight_normalization(getattr(self, "weight_normalization", "raw"))
        if current == mode:
            return new
        factor = self._normalization_denominator(current) / new._normalization_denominator(mode)
        new._eps_dev = new.epsilon_device * factor
        new._eps_host = None
        new.sfc_info["weight_normalization"] = mode
        new.sfc_info["field_integral"] = new._field_integral_for_normalization(mode)
        new.format_sfc_params()
        return new

    def to_unit_weight(self):
        if getattr(self, "field_kind", None) == "catalog_field":
            return self.switch_weight_normalization("field")
        total = getattr(self, "field_integral", None)
        if total is None:
            total = self._derived_field_integral(self)
        if total is None or not np.isfinite(total) or np.isclose(total, 0.0):
            raise ValueError("Cannot rescale a derived field with zero or non-finite epsilon sum.")
        new = self.copy()
        new._eps_dev = new.epsilon_device / total
        self._mark_derived(new)
        new.format_sfc_params()
        return new

    def with_normalization(self, normalization=None):
        mode = normalize_field_value_normalization(normalization)
        if mode is None:
            return self
        if mode == "unit":
            return self.to_unit_weight()
        if getattr(self, "field_kind", None) != "catalog_field":
            raise ValueError("normalization='raw', 'catalog', or 'field' can only be applied to catalog fields.")
        return self.switch_weight_normalization(mode)

    def switch_normalization(self, weight_normalization):
        return self.with_normalization(weight_normalization)

    def _resolve_value_unit(self, value_unit, sample_field=None):
        field = self if sample_field is None else sample_field
        value_unit = str(value_unit).strip().lower()
        if value_unit not in {"auto", "grid", "physical"}:
            raise ValueError("value_unit must be 'auto', 'grid', or 'physical'.")
        if value_unit == "auto":
            value_unit = "physical" if getattr(field, "field_kind", None) == "catalog_field" else "grid"
        return value_unit

    def phi_at_pos(self, pos):
        """Cell and scaling-function stencil of each position
        (io/sfc_field.py:484-485, utils/wavelet_grid.py:121-140): the cell
        floor(x * L / box) as int32 [N, 3], and float64 [N, 3, 3, 3] with
        phi_x * phi_y * phi_z at stencil offset s stored at index -s per
        axis (s = 0, 1, 2 -> 0, 2, 1), on the field's device."""
        support, res = int(self.phi_support), int(self.phi_resolution)
        dev = self.device if self.device is not None else "cpu"
        p = torch.as_tensor(np.asarray(pos, dtype=np.float64), device=dev) * float(self.scale_factor)
        coarse = torch.floor(p).to(torch.int32)
        frac = ((p - coarse.double()) * res).to(torch.int64)
        phi = torch.as_tensor(np.asarray(self.phi_array, dtype=np.float64), device=dev)
        taps = phi[frac[:, :, None] + torch.arange(support, device=dev) * res]  # [N, 3 axes, support]
        local = (taps[:, 0, :, None, None] * taps[:, 1, None, :, None]) * taps[:, 2, None, None, :]
        # out[:, i] holds offset (-i) mod support on every axis
        perm = torch.tensor([(-i) % support for i in range(support)], device=dev)
        out = local.index_select(1, perm).index_select(2, perm).index_select(3, perm)
        return coarse.cpu().numpy(), out.cpu().numpy()

    def field_density_at_pos(self, pos, epsilon=None, filter=None, normalization=None, value_unit="auto"):
        """pyhermes/io/sfc_field.py:487-530: the field's density at positions
        (box coordinates), by the 27-point scaling-function interpolation of
        utils/wavelet_grid.py:143-186 on the GPU (hermes_interp; float32
        gathers and products, float64 indices and output).  filter: a
        WindowFunc applied first; epsilon: an explicit coefficient grid."""
        import torch

        from .mc3pcf import interp

        if epsilon is not None and normalization is not None:
            raise ValueError("normalization cannot be applied when an explicit epsilon array is provided.")
        sample_field = self.with_normalization(normalization)
        value_unit = self._resolve_value_unit(value_unit, sample_field=sample_field)
        if epsilon is None:
            grid = (sample_field @ filter).epsilon_device if filter is not None else sample_field.epsilon_device
        else:
            grid = torch.as_tensor(np.asarray(epsilon) if not isinstance(epsilon, torch.Tensor) else epsilon,
                                   device=self.device)
        grid = grid.to(torch.float32).contiguous()
        L = int(sample_field.L)
        if tuple(grid.shape) != (L, L, L):
            raise ValueError(f"epsilon must have shape {(L, L, L)}, got {tuple(grid.shape)}.")
        phi = getattr(sample_field, "phi_array", None)
        if phi is None:
            from .phi import sample_scaling_function

            phi = sample_scaling_function()
        phi_t = torch.as_tensor(np.asarray(phi, dtype=np.float64), device=grid.device)
        p = torch.as_tensor(np.asarray(pos, dtype=np.float64) if not isinstance(pos, torch.Tensor) else pos,
                            dtype=torch.float64, device=grid.device)
        if p.ndim != 2 or p.shape[1] != 3:
            raise ValueError("pos must have shape (n, 3).")
        scaled = (p * float(sample_field.scale_factor)).contiguous()
        nx = interp(grid, int(round(math.log2(L))), scaled, phi_t).cpu().numpy()
        if value_unit == "physical":
            return nx * float(sample_field.scale_factor) ** 3
        return nx

    def field_mean_density(self, normalization=None, value_unit="auto"):
        """pyhermes/io/sfc_field.py:416-423."""
        field = self if normalization is None else self.with_normalization(normalization)
        value_unit = self._resolve_value_unit(value_unit, sample_field=field)
        value = getattr(field, "field_integral", None)
        if value is None:
            return None
        volume = float(field.V) if value_unit == "grid" else float(field.box_size) ** 3
        return value / volume

    # ---- persistence (byte-compatible with the reference) -------------------
    def save(self, f_out, save_sfc_field=False, save_counting=False, save_2pcf=False, save_3pcf=False,
             save_3pcf_multipole=False, single=True, overwrite=False):
        """io/base.py:90-124: the flag picks the writer; a field object
        writes its field file, and returns the path written (or None)."""
        if save_counting or save_2pcf or save_3pcf or save_3pcf_multipole:
            raise ValueError(f"{type(self).__name__} holds no counting / correlation results to save.")
        return self.save_sfc_field(f_out, single=single, overwrite=overwrite)

    def load(self, f_in, read_sfc_field=False, read_counting=False, read_2pcf=False, read_3pcf=False,
             read_3pcf_multipole=False, single=True):
        """io/base.py:24-88 for a field object: reads a field file."""
        if read_counting or read_2pcf or read_3pcf or read_3pcf_multipole:
            raise ValueError(f"{type(self).__name__} reads field files only.")
        self.load_sfc_field(f_in, single=single)

    def save_sfc_field(self, f_out, single=True, overwrite=False):
        """pyhermes/io/sfc_field.py:565-584: {'sfc_info', 'epsilon'} framed
        pickle, at the path check_fout resolves (returned)."""
        if not self.sfc_info:
            raise ValueError('The dictionary "sfc_info" is empty.')
        f_out = check_fout(self, f_out, overwrite)
        if f_out:
            with open(f_out, "wb") as f:
                write_numpy_pickle(f, {"sfc_info": self.sfc_info, "epsilon": self.epsilon})
        return f_out

    def load_sfc_field(self, f_in, single=True):
        """pyhermes/io/sfc_field.py:549-563."""
        with open(f_in, "rb") as f:
            dataset = read_numpy_pickle(f)
        if "epsilon" not in dataset:
            raise ValueError("Failed to load the dataset. The file is missing the 'epsilon' key.")
        self.epsilon = dataset["epsilon"]
        info = dataset.get("sfc_info")
        if info:
            self.sfc_info.update(info)
        self.format_sfc_params()
