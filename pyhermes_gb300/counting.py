"""``Counting``: the field density at uniformly random box positions.

Mirrors pyhermes/theory/counting.py (single process): the same parameters
(sfc_field, random_count, seed, weight_normalization = 'catalog', window,
threads, fout_path), the same positions (``default_rng(seed)`` uniform in
[0, box), utils/sampling.py:6-10; rank 0 of the reference), the field
optionally convolved with `window` first (:156-175), and
``nx = field_density_at_pos(pos, value_unit='physical')`` (:233) evaluated on
the GPU.  ``CountingData`` saves the reference's framed pickle
{'sfc_info', 'counting_info', 'nx'} (io/counting.py:47-62).
"""

import logging
import time

import numpy as np

from .params import task_params
from .sfc_field import (ResultFileIO, SFCField, check_fout, describe_input, normalize_task_weight_normalization,
                        read_numpy_pickle, write_numpy_pickle)
from .window import WindowFunc

logger = logging.getLogger("pyhermes_gb300.Counting")


def random_box_positions(count, box_size, ndim=3, rng=None, seed=None):
    """utils/sampling.py:6-10."""
    if rng is None:
        rng = np.random.default_rng(seed=seed)
    return rng.uniform(0.0, box_size, size=(count, ndim))


class CountingData(ResultFileIO):
    """Result container (pyhermes/io/counting.py:9-62)."""

    _OWN_SAVE, _OWN_LOAD = "save_counting", "load_counting"

    def __init__(self, data_path=None):
        self.sfc_info = {}
        self.counting_info = {}
        self.nx = None
        if data_path:
            self.load_counting(data_path)

    def save_counting(self, f_out, overwrite=False):
        if not self.counting_info:
            raise ValueError('The dictionary "counting_info" is empty.')
        f_out = check_fout(self, f_out, overwrite)
        if not f_out:
            return None
        with open(f_out, "wb") as f:
            write_numpy_pickle(f, {"sfc_info": self.sfc_info, "counting_info": self.counting_info, "nx": self.nx})
        return f_out

    def load_counting(self, f_in):
        with open(f_in, "rb") as f:
            dataset = read_numpy_pickle(f)
        if "nx" not in dataset:
            raise ValueError("Failed to load the dataset. The file is missing the 'nx' key.")
        self.nx = dataset["nx"]
        self.sfc_info = dataset.get("sfc_info") or {}
        self.counting_info.update(dataset.get("counting_info") or {})


class Counting:
    """GPU mirror of pyhermes.theory.counting.Counting."""

    def __init__(self, param_task=None, device="cuda"):
        self.task_params = task_params("Counting", param_task or {"Counting": {}})
        self.device = device
        self.format_params()

    def format_params(self):
        """The task parameters into attributes (theory/counting.py:28-40);
        call again after editing task_params."""
        p = self.task_params
        self.sfc_field = p.get("sfc_field", "")
        self._sfc_input = self.sfc_field
        self.random_count = int(p["random_count"])
        self.seed = int(p["seed"])
        self.weight_normalization = normalize_task_weight_normalization(p.get("weight_normalization", "catalog"))
        window = p.get("window", None)
        self.window = window if (window and (isinstance(window, WindowFunc) or window.get("type"))) else None
        self.threads = int(p.get("threads", 1))
        self.fout_path = p.get("fout_path", "")
        self._fields_prepared = False
        self.counting_data = CountingData()

    def _snapshot(self):
        # a window as theory/counting.py:89-100 records it
        return {"sfc_field": describe_input(self._sfc_input), "random_count": self.random_count, "seed": self.seed,
                "weight_normalization": self.weight_normalization, "window": describe_input(self.window),
                "threads": self.threads, "fout_path": self.fout_path}

    def prepare_input_fields(self, sfc_field=None, window=None):
        sfc_field = self.sfc_field if sfc_field is None else sfc_field
        window = self.window if window is None else window
        if isinstance(sfc_field, str):
            if not sfc_field:
                raise ValueError("No input 'sfc_field' provided.")
            base = SFCField(data_path=sfc_field, device=self.device)
        elif isinstance(sfc_field, SFCField):
            base = sfc_field
        else:
            raise TypeError("'sfc_field' must be a string path or a SFCField instance.")
        if window is not None and not isinstance(window, WindowFunc):
            if not isinstance(window, dict):
                raise TypeError(f"Unsupported window input. Expected dict, WindowFunc, or None, got {type(window)}.")
            window = WindowFunc(window, base.sfc_info, device=self.device)
        if self.weight_normalization != "unit" and getattr(base, "field_kind", None) == "catalog_field":
            base = base.with_normalization(self.weight_normalization)
        elif self.weight_normalization == "unit":
            base = base.with_normalization("unit")
        self.sfc_field = base @ window if window is not None else base
        self.window = window
        self.counting_data.counting_info = self._snapshot()
        self.counting_data.sfc_info = self.sfc_field.sfc_info
        self._fields_prepared = True

    def run(self, save_result=True, overwrite=False):
        t0 = time.perf_counter()
        if not self._fields_prepared:
            self.prepare_input_fields()
        pos = random_box_positions(self.random_count, self.sfc_field.box_size, seed=self.seed)
        self.counting_data.nx = np.asarray(self.sfc_field.field_density_at_pos(pos, value_unit="physical"),
                                           dtype=np.float64)
        self.counting_data.counting_info = self._snapshot()
        if save_result and self.fout_path:
            self.counting_data.save_counting(self.fout_path, overwrite=overwrite)
        logger.info("Counting %d positions in %.4f s", self.random_count, time.perf_counter() - t0)
        return self.counting_data
