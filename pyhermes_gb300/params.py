"""Task parameter defaults and merging, mirroring the reference's
``TaskBase`` + ``ParamBase.recursive_update`` behaviour
(pyhermes/pipeline/pipeline.py:12-49, pyhermes/param/parambase.py:116-172):
a user dict ``{TaskName: {...}}`` is merged into the task defaults; keys in
``REPLACE_KEYS`` are replaced wholesale instead of merged.

The defaults restate the values of the reference's per-package
default_params.json files for the keys this package reads.
"""

import copy

import numpy as np

_ATOMIC = (str, int, float, bool, complex, type(None), np.generic)


def plain_copy(obj):
    """``copy.deepcopy`` for parameter structures, without its memo
    bookkeeping: plain dict / list / tuple containers are rebuilt, numpy
    arrays copied, immutable scalars shared; anything else goes through
    ``copy.deepcopy`` (which shares functions, as before)."""
    if isinstance(obj, _ATOMIC):
        return obj
    t = type(obj)
    if t is dict:
        return {k: plain_copy(v) for k, v in obj.items()}
    if t is list:
        return [plain_copy(v) for v in obj]
    if t is tuple:
        return tuple(plain_copy(v) for v in obj)
    if t is np.ndarray:
        return obj.copy()
    return copy.deepcopy(obj)


def callable_metadata(value):
    """A callable as result files record it (utils/window_params.py:97-101):
    {'kind': 'callable', 'name': '<module>.<qualname>'} (a numba dispatcher
    is named by its Python function)."""
    target = getattr(value, "py_func", value)
    module = getattr(target, "__module__", getattr(value, "__module__", type(value).__module__))
    name = getattr(target, "__qualname__", getattr(target, "__name__", type(value).__name__))
    return {"kind": "callable", "name": f"{module}.{name}"}


def serialize_window_params(value):
    """Window / sampling parameters as result files record them
    (utils/window_params.py:104-121): 'func' becomes 'custom_func' metadata,
    other callables their metadata, arrays lists, NumPy scalars Python ones."""
    if isinstance(value, dict):
        return {("custom_func" if k == "func" else k): (callable_metadata(v) if k == "func"
                                                         else serialize_window_params(v))
                for k, v in value.items()}
    if callable(value):
        return callable_metadata(value)
    if isinstance(value, np.ndarray):
        return value.tolist()
    if isinstance(value, (list, tuple)):
        return [serialize_window_params(v) for v in value]
    if isinstance(value, np.generic):
        return value.item()
    return copy.deepcopy(value)


REPLACE_KEYS = {
    "Corr_2PCF.binning_window",
    "Corr_2PCF.sampling",
    "Corr_3PCF_Multipole.binning_window12",
    "Corr_3PCF_Multipole.binning_window13",
    "Corr_3PCF_Multipole.sampling",
    "Corr_3PCF_Multipole.sample_mpi",
}

def _empty_window():
    # a fresh nested dict per key: task_params deep-copies the defaults, and
    # deepcopy keeps any sharing between them, so one shared inner len_args
    # dict would receive every window's arguments during the merge
    return {"type": "", "len_args": {}, "los_args": {}, "other_args": {}}

DEFAULTS = {
    "Counting": {
        "sfc_field": "",
        "random_count": 1000000,
        "seed": 42,
        "weight_normalization": "catalog",
        "window": _empty_window(),
        "threads": 1,
        "fout_path": "",
    },
    "SFCProjection": {
        "fin": {"path": "", "format": "bin",
                "download": {"cache_path": "", "cache_dir": "", "sha256": "", "timeout": 60},
                "reader_params": {"dtype": "float32", "ncols": 3, "pos_cols": [0, 1, 2], "fields": {}},
                "catalog_weight_key": None, "field_value_key": None},
        "particle_pos": None,
        "catalog_weight": None,
        "field_value": None,
        "weight_normalization": "catalog",
        "box_size": 1000,
        "J": 8,
        "wavelet_mode": "db2",
        "wavelet_level": 10,
        "phi_resolution": 1024,
        "save_particle_data": False,
        "particle_data_path": "",
        "threads": 1,
        "fout_path": "",
    },
    "Corr_2PCF": {
        "sfc_field": "", "sfc_field1": "", "sfc_field2": "",
        "random": None, "random1": "", "random2": "",
        "weight_normalization": "catalog",
        "window": _empty_window(), "window1": _empty_window(), "window2": _empty_window(),
        "binning_window": {"type": "shell", "len_args": ["R"], "los_args": {}, "other_args": {},
                           "mapping": "s_to_R", "kernel_mode": ""},
        "sampling": {"s": {"min": 1.0, "max": 150.0, "n": 30}},
        "threads": 1,
        "products": "xi",
        "memory_strategy": "speed",
        "binning_window_cache": False,
        "binning_window_cache_dir": "",
        "fout_path": "",
    },
    "Corr_3PCF_Multipole": {
        "sfc_field": "", "sfc_field1": "", "sfc_field2": "", "sfc_field3": "",
        "random": None, "random1": "", "random2": "", "random3": "",
        "weight_normalization": "catalog",
        "window": _empty_window(), "window1": _empty_window(),
        "window2": _empty_window(), "window3": _empty_window(),
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {}},
        "sampling": {},
        "l_min": 0,
        "l_max": 4,
        "gpu_device_id": 0,
        "gpu_threads_per_block": [8, 8, 8],
        "summation_backend": "gb300",
        "execution_mode": "serial",
        "sample_mpi": {"ranks_per_sample": 1, "gpu_device_ids": []},
        "cache_multipole_fields": False,
        "cache_dir": "",
        "verbose_m_progress": False,
        "verbose_profile": False,
        "zeta_condition_warning": 1.0e12,
        "threads": 1,
        "products": "zeta_l",
        "fout_path": "",
        "contraction_engine": "tensor",
    },
    "Corr_3PCF": {
        "sfc_field": "", "sfc_field1": "", "sfc_field2": "", "sfc_field3": "",
        "particle_pos1": None, "particle_weight1": None, "random_pos1": None, "random_weight1": None,
        "random": None, "random1": "", "random2": "", "random3": "",
        "weight_normalization": "catalog",
        "window": _empty_window(), "window1": _empty_window(),
        "window2": _empty_window(), "window3": _empty_window(),
        "r12": 20.0, "r13": 40.0,
        "angle_param": "theta",
        "theta": {"theta_min": 0.0, "theta_max": 3.141592653589793, "n_theta": 20},
        "mu": {"mu_min": -1.0, "mu_max": 1.0, "n_mu": 20},
        "n_rot": 100,
        "center": "box_random",
        "n_box_centers": 5000000,
        "base_seed": 42,
        "threads": 1,
        "products": "Q",
        "fout_path": "",
    },
}


def _is_array_like(v):
    return hasattr(v, "shape") and hasattr(v, "dtype")


def recursive_update(default, new, section):
    """Merge ``new`` into ``default`` in place (REPLACE_KEYS replaced whole)."""
    for key, value in new.items():
        path = f"{section}.{key}"
        if (isinstance(value, dict) and isinstance(default.get(key), dict)
                and path not in REPLACE_KEYS):
            recursive_update(default[key], value, path)
        else:
            default[key] = value if _is_array_like(value) else copy.deepcopy(value)
    return default


def task_params(task_name, param_task):
    """Return the merged parameter dict for ``task_name``."""
    if param_task is None:
        param_task = {task_name: {}}
    if task_name not in param_task:
        raise ValueError(
            f"Mismatch of task name, expected <{task_name}>, but it was not found in "
            f"the provided task(s) <{list(param_task)}>"
        )
    merged = copy.deepcopy(DEFAULTS[task_name])
    return recursive_update(merged, param_task[task_name], task_name)
