"""``Corr_2PCF``: two-point correlation of SFC fields on one GB300.

Mirrors ``pyhermes/theory/corr2pcf.py`` (speed strategy, single process):
the same parameter dict, products dd / dr / rd / delta_dd / rr / xi
(:27-42), sampling grids and binning-window mappings s_to_R, smu_to_RH,
rppi_to_RH or a callable (:267-315), task weight normalisation (:606-629),
optional vertex windows (``field @ window``), the uniform-random shortcut
(:355-363, :1022-1032) and the physical rescale by scale_factor**6
(:594-604).

Difference by design: the reference builds one kernel and runs two FFTs per
sample and product (pair_product_with_window, :366-372).  Here each
distinct field is transformed once, and every sample's pair products come
from one pass over the half spectra (Parseval), with the binning kernels
evaluated on the fly (``hermes_pair_products``).  The k = 0 term of
mean-subtracted fields is added on the host in float64.
"""

import copy
import itertools
import logging
import time

import numpy as np
import torch

from .params import plain_copy, task_params
from .sfc_field import (ResultFileIO, SFCField, check_fout, describe_input, normalize_task_weight_normalization,
                        read_numpy_pickle, write_numpy_pickle)
from .window import (
    ANISOTROPIC_AUTO_WINDOW_TYPES, LOS_AWARE_WINDOW_TYPES, WindowFunc, materialized_pair_products, normalize_los_args,
    pair_products, rfft_field,
)

logger = logging.getLogger("pyhermes_gb300.Corr_2PCF")

PRODUCT_NAMES = ("dd", "dr", "rd", "delta_dd", "rr", "xi")
PRODUCT_DEPS = {"xi": ["delta_dd", "rr"]}
NONNEGATIVE_SAMPLING_ARGS = {"s", "rp", "pi"}
BUILTIN_BINNING_WINDOW_TYPES = {"shell", "thick_shell"} | ANISOTROPIC_AUTO_WINDOW_TYPES


def normalize_products(products):
    """theory/corr2pcf.py:53-73."""
    if isinstance(products, str):
        products = [products]
    elif products is None:
        products = ["xi"]
    out = []
    for item in products:
        name = str(item).strip().lower()
        if name not in PRODUCT_NAMES:
            raise ValueError(f"Unsupported product '{item}'. Allowed values are {sorted(PRODUCT_NAMES)}.")
        if name not in out:
            out.append(name)
    return out


def expand_products(products):
    out = list(products)
    i = 0
    while i < len(out):
        for d in PRODUCT_DEPS.get(out[i], []):
            if d not in out:
                out.append(d)
        i += 1
    return out


def normalize_sampling_spec(name, spec):
    """theory/corr2pcf.py:217-231 and :87-98."""
    nonneg = name in NONNEGATIVE_SAMPLING_ARGS
    if isinstance(spec, dict):
        n = int(spec["n"])
        if n <= 0:
            raise ValueError(f"'{name}' sampling n must be positive.")
        arr = np.linspace(float(spec["min"]), float(spec["max"]), n, dtype=np.float64)
    else:
        arr = np.asarray(spec, dtype=np.float64)
        if arr.ndim != 1 or arr.size == 0:
            raise ValueError(f"'{name}' must be a non-empty 1D array-like input.")
        d = np.diff(arr)
        if np.any(d < 0.0) and np.any(d > 0.0):
            raise ValueError(f"'{name}' values must be monotonic.")
    if nonneg and np.any(arr < 0.0):
        raise ValueError(f"'{name}' sampling values must be non-negative.")
    return np.ascontiguousarray(arr, dtype=np.float64)


def mapping_s_to_R(sample, bw):
    p = plain_copy(bw)
    p.setdefault("len_args", {})
    if p["len_args"].get("R") is None:
        p["len_args"]["R"] = sample["s"]
    return p


def mapping_smu_to_RH(sample, bw):
    p = plain_copy(bw)
    p.setdefault("len_args", {})
    if p["len_args"].get("R") is None:
        p["len_args"]["R"] = sample["s"] * np.sqrt(max(0.0, 1.0 - sample["mu"] * sample["mu"]))
    if p["len_args"].get("H") is None:
        p["len_args"]["H"] = sample["s"] * sample["mu"]
    return p


def mapping_rppi_to_RH(sample, bw):
    p = plain_copy(bw)
    p.setdefault("len_args", {})
    if p["len_args"].get("R") is None:
        p["len_args"]["R"] = sample["rp"]
    if p["len_args"].get("H") is None:
        p["len_args"]["H"] = sample["pi"]
    return p


BINNING_WINDOW_MAPPING_SPECS = {
    "s_to_R": {"sampling_args": ("s",), "func": mapping_s_to_R},
    "smu_to_RH": {"sampling_args": ("s", "mu"), "func": mapping_smu_to_RH},
    "rppi_to_RH": {"sampling_args": ("rp", "pi"), "func": mapping_rppi_to_RH},
}


def _normalize_len_args(len_args):
    if len_args is None:
        return {}
    if isinstance(len_args, dict):
        return copy.deepcopy(len_args)
    if isinstance(len_args, str):
        return {len_args: None}
    return {item: None for item in len_args}


def normalize_binning_window(bw):
    """utils/window_params.py:124-189 (+ corr2pcf.py:318-332)."""
    if bw is None:
        bw = {"type": "shell", "len_args": {"R": None}, "los_args": {}, "other_args": {},
              "mapping": "s_to_R", "kernel_mode": "octant"}
    elif isinstance(bw, str):
        t = bw.strip().lower()
        if t not in BUILTIN_BINNING_WINDOW_TYPES:
            raise ValueError(f"Unsupported binning_window string '{bw}'.")
        bw = {"type": t}
    p = copy.deepcopy(bw)
    t = str(p.get("type", "shell")).strip().lower()
    p["type"] = t
    if t == "shell":
        p["len_args"] = {**{"R": None}, **_normalize_len_args(p.get("len_args", {}))}
        p.setdefault("mapping", "s_to_R")
    elif t == "thick_shell":
        la = _normalize_len_args(p.get("len_args", {}))
        la.setdefault("R", None)
        la.setdefault("delta_R", None)
        p["len_args"] = la
        p.setdefault("mapping", "s_to_R")
    elif t in LOS_AWARE_WINDOW_TYPES:
        la = _normalize_len_args(p.get("len_args", {}))
        la.setdefault("R", None)
        la.setdefault("H", None)
        p["len_args"] = la
        p.setdefault("los_args", {"nx": 0.0, "ny": 0.0, "nz": 1.0})
        p.setdefault("mapping", "smu_to_RH")
    p["len_args"] = _normalize_len_args(p.get("len_args", {}))
    p["los_args"] = normalize_los_args(p.get("los_args", {}), t)
    p.setdefault("other_args", {})
    km = p.get("kernel_mode")
    if not km:
        km = "auto" if t in ANISOTROPIC_AUTO_WINDOW_TYPES else ("complex_rfft" if t == "directional_derivative"
                                                                else "octant")
    p["kernel_mode"] = km
    mapping = p.get("mapping")
    if isinstance(mapping, str) and mapping not in BINNING_WINDOW_MAPPING_SPECS:
        raise ValueError(f"Unsupported binning_window mapping '{mapping}'.")
    return p


def build_binning_window_params_for_sample(sample, bw):
    mapping = bw.get("mapping")
    mapper = BINNING_WINDOW_MAPPING_SPECS[mapping]["func"] if isinstance(mapping, str) else mapping
    params = mapper(sample, bw)
    if not isinstance(mapping, str):  # the built-in mappings already return a fresh copy
        params = plain_copy(params)
    params.pop("mapping", None)
    params.setdefault("len_args", {})
    params.setdefault("los_args", {})
    params.setdefault("other_args", {})
    return params


def compute_pair_product_at_sample(sample, sfc_field1, sfc_field2=None, binning_window=None):
    """One pair product in grid units at one sample (theory/corr2pcf.py:
    375-382): the product of mean densities when a vertex is a scalar, else
    the mean over cells of (field1 convolved with the sample's binning
    window) * field2, on the GPU."""
    if sfc_field2 is None:
        sfc_field2 = sfc_field1
    if _is_scalar(sfc_field1) or _is_scalar(sfc_field2):
        return field_mean_density(sfc_field1) * field_mean_density(sfc_field2)
    params = build_binning_window_params_for_sample(sample, normalize_binning_window(binning_window))
    window = WindowFunc(params, sfc_field1.sfc_info, threads=getattr(sfc_field1, "threads", None),
                        device=sfc_field1.device)
    e1 = sfc_field1.epsilon_device.to(torch.float32).contiguous()
    e2 = e1 if sfc_field2 is sfc_field1 else sfc_field2.epsilon_device.to(torch.float32).contiguous()
    if window.materialized:
        v, _ = materialized_pair_products([e1, e2], [(0, 1)], [window], exclude_k0=False)
        return float(v[0, 0])
    if window.resolved_mode() == "complex_full_fft":
        raise ValueError("A complex full-FFT window has no rFFT pair product.")
    s1 = rfft_field(e1)
    specs, pair = ([s1], (0, 0)) if e2 is e1 else ([s1, rfft_field(e2)], (0, 1))
    v, k0 = pair_products(specs, [pair], [window], exclude_k0=True)
    # the k = 0 term in float64
    dc1 = float(e1.double().sum().item())
    dc2 = dc1 if e2 is e1 else float(e2.double().sum().item())
    return float(v[0, 0] + dc1 * dc2 * k0[0] / float(e1.shape[0]) ** 6)


class Corr2PCFData(ResultFileIO):
    """Result container (pyhermes/io/corr2pcf.py): sampling + products.

    The file written by ``save_corr2pcf`` / read by ``load_corr2pcf`` is the
    reference's NumPy-framed pickle with the same top-level keys and order:
    sfc_info1, sfc_info2, corr2pcf_info, sampling_names, the products
    dd .. xi, then one array per sampling name."""

    _OWN_SAVE, _OWN_LOAD = "save_corr2pcf", "load_corr2pcf"

    def __init__(self, data_path=None):
        self.sampling_names = ()
        self.sampling = {}
        for p in PRODUCT_NAMES:
            setattr(self, p, None)
        self.corr2pcf_info = {}
        self.sfc_info1 = None
        self.sfc_info2 = None
        if data_path:
            self.load_corr2pcf(data_path)

    def set_sampling(self, names, arrays):
        self.sampling_names = tuple(names)
        self.sampling = dict(arrays)
        for n, a in arrays.items():
            setattr(self, n, a)

    def save_corr2pcf(self, f_out, overwrite=False):
        f_out = check_fout(self, f_out, overwrite)
        if not f_out:
            return None
        data = {"sfc_info1": self.sfc_info1, "sfc_info2": self.sfc_info2, "corr2pcf_info": self.corr2pcf_info,
                "sampling_names": tuple(self.sampling_names)}
        data.update({p: getattr(self, p) for p in PRODUCT_NAMES})
        data.update({n: self.sampling[n] for n in self.sampling_names})
        with open(f_out, "wb") as f:
            write_numpy_pickle(f, data)
        return f_out

    def load_corr2pcf(self, f_in):
        with open(f_in, "rb") as f:
            d = read_numpy_pickle(f)
        names = tuple(d.get("sampling_names") or ())
        self.set_sampling(names, {n: d[n] for n in names if n in d})
        for p in PRODUCT_NAMES:
            setattr(self, p, d.get(p))
        self.corr2pcf_info = d.get("corr2pcf_info") or {}
        self.sfc_info1 = d.get("sfc_info1")
        self.sfc_info2 = d.get("sfc_info2")


def _is_scalar(v):
    return isinstance(v, (float, int, np.floating))


def field_mean_density(field, value_unit="grid"):
    if _is_scalar(field):
        return float(field)
    value = field.field_mean_density(value_unit=value_unit)
    if value is None:
        raise ValueError("Cannot extract a uniform density from a field without field_integral metadata.")
    return value


class Corr_2PCF:
    task_name = "Corr_2PCF"

    def __init__(self, param_task=None, device="cuda"):
        self.task_params = task_params(self.task_name, param_task)
        self.device = torch.device(device)
        self.rank, self.size = 0, 1
        self.format_params()

    def format_params(self):
        """The task parameters into attributes (theory/corr2pcf.py:419-470); call again after
        editing task_params."""
        tp = self.task_params
        self.sfc_field = tp.get("sfc_field", "")
        self.sfc_field1 = tp.get("sfc_field1", "") or self.sfc_field
        self.sfc_field2 = tp.get("sfc_field2", "") or self.sfc_field
        self.random = tp.get("random", None)
        self.random1 = tp.get("random1") if tp.get("random1") not in (None, "") else self.random
        self.random2 = tp.get("random2") if tp.get("random2") not in (None, "") else self.random
        self.weight_normalization = normalize_task_weight_normalization(tp.get("weight_normalization", "catalog"))
        window = tp.get("window")
        self.window = window if (window and window.get("type")) else None
        for i in (1, 2):
            wi = tp.get(f"window{i}")
            wi = wi if (wi and wi.get("type")) else None
            if not wi and self.window:
                wi = dict(self.window)
            setattr(self, f"window{i}", wi)
        self.binning_window = normalize_binning_window(tp.get("binning_window"))
        self.sampling = copy.deepcopy(tp["sampling"])
        self.products = normalize_products(tp.get("products", "xi"))
        self.threads = int(tp.get("threads", 1))
        self.fout_path = tp.get("fout_path", "")
        self._fields_prepared = False

    def _info_snapshot(self):
        """corr2pcf_info with the reference's keys (theory/corr2pcf.py:919-1112,
        _current_task_params_snapshot): inputs summarised, randoms resolved."""
        rand = getattr(self, "rand", {}) or {}
        info = {"sfc_field": describe_input(self.sfc_field), "sfc_field1": describe_input(self.sfc_field1),
                "sfc_field2": describe_input(self.sfc_field2), "random": describe_input(self.random)}
        for i in (1, 2):
            info[f"random{i}"] = describe_input(rand.get(i, getattr(self, f"random{i}")))
        info.update({"window": describe_input(self.window), "window1": describe_input(self.window1),
                     "window2": describe_input(self.window2),
                     "binning_window": {k: v for k, v in self.binning_window.items()
                                        if k != "mapping" or isinstance(v, str)},
                     "sampling_spec": plain_copy(self.sampling), "sampling_names": list(self.sampling_names),
                     "sampling": {n: [float(v) for v in self.sampling_arrays[n]] for n in self.sampling_names},
                     "threads": self.threads, "products": list(self.products), "memory_strategy": "speed",
                     "binning_window_cache": False, "binning_window_cache_dir": "",
                     "weight_normalization": self.weight_normalization, "fout_path": self.fout_path})
        return info

    # ---- sampling ----------------------------------------------------------
    def _resolve_sampling(self):
        if not isinstance(self.sampling, dict) or not self.sampling:
            raise ValueError("Corr_2PCF requires a non-empty 'sampling' dictionary.")
        mapping = self.binning_window.get("mapping")
        required = (BINNING_WINDOW_MAPPING_SPECS[mapping]["sampling_args"] if isinstance(mapping, str)
                    else tuple(self.sampling.keys()))
        missing = [n for n in required if n not in self.sampling]
        extra = [n for n in self.sampling if n not in required]
        if missing or extra:
            raise ValueError(f"sampling keys must match mapping '{mapping}': expected {list(required)}, "
                             f"missing={missing}, extra={extra}.")
        self.sampling_names = tuple(required)
        self.sampling_arrays = {n: normalize_sampling_spec(n, self.sampling[n]) for n in required}

    # ---- inputs ---------------------------------------------------------------
    def _resolve_field(self, value, what):
        if isinstance(value, SFCField):
            return value
        if isinstance(value, str) and value:
            return SFCField(data_path=value, threads=self.threads, device=self.device)
        raise ValueError(f"Missing usable input for {what}: expected a path or SFCField.")

    def _field_in_task_normalization(self, field):
        self._density_physical_scale = float(field.scale_factor) ** 3
        if self.weight_normalization == "unit":
            return field.with_normalization("unit")
        if getattr(field, "field_kind", None) != "catalog_field":
            return field.copy()
        return field.switch_weight_normalization(self.weight_normalization)

    def _required_flags(self):
        flags = {"dd": (True, False), "dr": (True, True), "rd": (True, True), "delta_dd": (True, True),
                 "rr": (False, True), "xi": (True, True)}
        nd = nr = False
        for p in expand_products(self.products):
            a, b = flags[p]
            nd, nr = nd or a, nr or b
        return nd, nr

    def _apply_window(self, field, win):
        if win is None:
            out = field.copy()
            out.format_sfc_params()
            return out
        w = win if isinstance(win, WindowFunc) else WindowFunc(win, field.sfc_info, threads=self.threads,
                                                                device=self.device)
        return field @ w

    def prepare_input_fields(self):
        self._resolve_sampling()
        needs_data, needs_random = self._required_flags()
        self.data = {}
        self.rand = {}
        for i in (1, 2):
            win = getattr(self, f"window{i}")
            if needs_data:
                base = self._field_in_task_normalization(self._resolve_field(getattr(self, f"sfc_field{i}"),
                                                                             f"field vertex {i}"))
                self.data[i] = self._apply_window(base, win)
            if needs_random:
                r = getattr(self, f"random{i}")
                if r is None or r == "":
                    raise ValueError(f"Missing input for random vertex {i}. Products {self.products} require "
                                     f"'random{i}' or shared 'random'.")
                if r == "uniform":
                    ref = self.data.get(i)
                    if ref is None:
                        ref = self._field_in_task_normalization(self._resolve_field(getattr(self, f"sfc_field{i}"),
                                                                                    f"field vertex {i}"))
                    if ref.field_mean_density(value_unit="grid") is None:
                        raise ValueError("random='uniform' requires a SFCField field with a defined field_integral.")
                    self.rand[i] = field_mean_density(ref)
                else:
                    base = self._field_in_task_normalization(self._resolve_field(r, f"random vertex {i}"))
                    self.rand[i] = self._apply_window(base, win)
        self._fields_prepared = True

    # ---- products ---------------------------------------------------------------
    def calc_pair_product(self, sample, field1, field2=None, binning_window=None):
        """theory/corr2pcf.py:632-645: one pair product at one sample with
        the task's binning window (or the one given)."""
        return compute_pair_product_at_sample(sample, field1, field2,
                                              self.binning_window if binning_window is None else binning_window)

    def _binning_windows(self, ref_field):
        bws = []
        for idx in itertools.product(*(range(self.sampling_arrays[n].size) for n in self.sampling_names)):
            sample = {n: float(self.sampling_arrays[n][i]) for n, i in zip(self.sampling_names, idx)}
            params = build_binning_window_params_for_sample(sample, self.binning_window)
            bws.append(WindowFunc(params, ref_field.sfc_info, threads=self.threads, device=self.device))
        return bws

    def _binning_family(self, ref_field):
        """The bins as one template WindowFunc plus per-bin descriptors when
        every sample's window is the same built-in window with different
        len_args (the mappings of corr2pcf.py:267-315 only set lengths), else
        None (then every bin gets its own WindowFunc)."""
        from .window import family_descriptors

        params = []
        for idx in itertools.product(*(range(self.sampling_arrays[n].size) for n in self.sampling_names)):
            sample = {n: float(self.sampling_arrays[n][i]) for n, i in zip(self.sampling_names, idx)}
            params.append(build_binning_window_params_for_sample(sample, self.binning_window))
        rest = [{k: v for k, v in p.items() if k != "len_args"} for p in params]
        if any(r != rest[0] for r in rest[1:]):
            return None
        template = WindowFunc(params[0], ref_field.sfc_info, threads=self.threads, device=self.device)
        if template.materialized or template.has_custom_func or template.is_composite_window:
            return None
        try:
            template.descriptor()
        except ValueError:
            return None
        return template, family_descriptors(template, [p.get("len_args") or {} for p in params])

    @staticmethod
    def _dc(field):
        """float64 sum of a field (its k = 0 Fourier coefficient)."""
        return float(field.epsilon_device.double().sum().item())

    def run(self, save_result=True, overwrite=False):
        t0 = time.perf_counter()
        if not self._fields_prepared:
            self.prepare_input_fields()
        expanded = expand_products(self.products)
        computed = [p for p in expanded if p != "xi"]
        shape = tuple(self.sampling_arrays[n].size for n in self.sampling_names)
        ref = next((f for f in list(self.data.values()) + list(self.rand.values()) if isinstance(f, SFCField)),
                   None)
        results = {}
        # operands of each product: (a, b) with a, b in {"D1","D2","R1","R2","d1","d2"}
        operand = {"dd": ("D1", "D2"), "dr": ("D1", "R2"), "rd": ("R1", "D2"), "delta_dd": ("d1", "d2"),
                   "rr": ("R1", "R2")}

        def value_of(key):
            side = int(key[1])
            if key[0] == "D":
                return self.data[side]
            if key[0] == "R":
                return self.rand[side]
            return ("delta", side)

        field_keys, spectra, reals, dcs = {}, [], [], {}
        pairs, pair_products_of = [], {}
        scalar_results = {}
        for prod in computed:
            a, b = operand[prod]
            va, vb = value_of(a), value_of(b)
            if _is_scalar(va) or _is_scalar(vb):
                # corr2pcf.py:284-287: scalar vertices give mean-density products
                def dens(v, side):
                    if isinstance(v, tuple):
                        raise ValueError("delta of a uniform random is not a scalar")
                    return field_mean_density(v)
                scalar_results[prod] = dens(va, 1) * dens(vb, 2)
                continue
            keys = []
            for k in (a, b):
                side = int(k[1])
                if k[0] == "d" and not _is_scalar(self.rand[side]):
                    spec_key = k  # delta against a random field: transform D - R itself
                    fld_t = (self.data[side].epsilon_device.double()
                             - self.rand[side].epsilon_device.double()).to(torch.float32)
                else:
                    spec_key = k if k[0] != "d" else "D" + k[1]
                    fld = self.data[side] if spec_key[0] == "D" else self.rand[side]
                    fld_t = fld.epsilon_device.to(torch.float32)
                if spec_key not in field_keys:
                    field_keys[spec_key] = len(spectra)
                    spectra.append(rfft_field(fld_t.contiguous()))
                    reals.append(fld_t.contiguous())
                    dcs[spec_key] = float(fld_t.double().sum().item())
                keys.append(field_keys[spec_key])
            pair_products_of[prod] = len(pairs)
            pairs.append(tuple(keys))
        if pairs:
            family = self._binning_family(ref)
            if family is not None:
                # one built-in window family: descriptors without per-bin objects
                template, descs = family
                vals = np.zeros((len(descs), len(pairs)))
                k0 = np.zeros(len(descs))
                for s in range(0, len(pairs), 4):
                    v, kb = pair_products(spectra, pairs[s:s + 4], [template], exclude_k0=True, descs=descs)
                    vals[:, s:s + 4] = v
                    k0[:] = kb
                L = template.L
            else:
                windows = self._binning_windows(ref)
                # split into groups of <= 4 pairs per pass
                vals = np.zeros((len(windows), len(pairs)))
                k0 = np.zeros(len(windows))
                # built-in bins evaluate their kernels on the fly; bins with a
                # stored kernel (custom callables) go through the convolution
                on_fly = [b for b, w in enumerate(windows) if not w.materialized]
                stored = [b for b, w in enumerate(windows) if w.materialized]
                for s in range(0, len(pairs), 4):
                    if on_fly:
                        v, kb = pair_products(spectra, pairs[s:s + 4], [windows[b] for b in on_fly],
                                              exclude_k0=True)
                        vals[on_fly, s:s + 4] = v
                        k0[on_fly] = kb
                if stored:
                    v, kb = materialized_pair_products(reals, pairs, [windows[b] for b in stored], exclude_k0=True)
                    vals[stored, :] = v
                    k0[stored] = kb
                L = windows[0].L
            N2 = float(L) ** 6
            for prod, col in pair_products_of.items():
                a, b = operand[prod]

                def dc_of(k):
                    side = int(k[1])
                    if k[0] == "d":
                        r = self.rand[side]
                        if not _is_scalar(r):
                            return dcs[k]
                        return dcs["D" + k[1]] - float(r) * float(L) ** 3
                    return dcs[k]

                # the k = 0 term in float64 (mean-subtracted fields lose it in float32)
                results[prod] = (vals[:, col] + dc_of(a) * dc_of(b) * k0 / N2).reshape(shape)
        for prod, v in scalar_results.items():
            results[prod] = np.full(shape, v, dtype=np.float64)
        factor = float(getattr(self, "_density_physical_scale", 1.0)) ** 2
        if not np.isclose(factor, 1.0):
            for prod in ("dd", "dr", "rd", "delta_dd", "rr"):
                if prod in results:
                    results[prod] = results[prod] * factor
        data = Corr2PCFData()
        data.set_sampling(self.sampling_names, {n: self.sampling_arrays[n].copy() for n in self.sampling_names})
        for p in PRODUCT_NAMES:
            setattr(data, p, results.get(p) if p in expanded else None)
        if "xi" in expanded:
            data.xi = data.delta_dd / data.rr
        data.corr2pcf_info = self._info_snapshot()
        if 1 in self.data:
            data.sfc_info1 = self.data[1].sfc_info
        if 2 in self.data:
            data.sfc_info2 = self.data[2].sfc_info
        self.corr2pcf_data = data
        if save_result and self.fout_path:
            data.save_corr2pcf(self.fout_path, overwrite=overwrite)
        logger.info("Corr_2PCF %d samples in %.4f s", int(np.prod(shape)), time.perf_counter() - t0)
        return data
