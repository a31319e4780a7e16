"""``SFCProjection``: catalogue -> SFCField on one GB300.

Mirrors ``pyhermes/base/sfc_projection.py:64-419`` (single-process path):
the same parameter dict, float64 weight normalisation on the host
(:251-282), the same ``sfc_info`` keys (:381-403) and the same result
object.  The deposit itself is ``hermes_deposit`` (csrc/deposit.cu).
The MPI x-slab path (:325-379) has no counterpart: one process owns the GPU.
"""

import copy
import os
import logging
import time

import numpy as np
import torch

from . import kernels
from .params import task_params
from .phi import sample_scaling_function
from .sfc_field import SFCField, normalize_weight_normalization

logger = logging.getLogger("pyhermes_gb300.SFCProjection")


class SFCProjection:
    task_name = "SFCProjection"

    def __init__(self, param_task=None, device="cuda"):
        self.task_params = task_params(self.task_name, param_task)
        self.device = torch.device(device)
        self.rank, self.size = 0, 1
        self.format_params()
        self.sfc_field = None
        self._fields_prepared = False
        self._workspace = kernels.DepositWorkspace(self.device)

    def format_params(self):
        tp = self.task_params
        self.fin = copy.deepcopy(tp["fin"])
        self.particle_pos = tp["particle_pos"]
        self.catalog_weight = tp["catalog_weight"]
        self.field_value = tp["field_value"]
        self.weight_normalization = normalize_weight_normalization(tp.get("weight_normalization", "catalog"))
        self.box_size = tp["box_size"]
        self.J = int(tp["J"])
        self.L = 1 << self.J
        self.wavelet_mode = tp["wavelet_mode"]
        self.wavelet_level = tp["wavelet_level"]
        self.phi_resolution = int(tp["phi_resolution"])
        self.save_particle_data = bool(tp["save_particle_data"])
        self.particle_data_path = tp["particle_data_path"]
        self.threads = int(tp["threads"])
        self.fout_path = tp["fout_path"]

    def _read_catalogue(self):
        """Catalogue files (fin.path) are read by the caller: this package
        projects positions given as arrays (particle_pos, with optional
        catalog_weight / field_value)."""
        raise ValueError("SFCProjection needs particle_pos: read the catalogue file (fin.path) in the caller and pass "
                         "its positions, weights and values as arrays.")

    def _load_particle_input(self):
        """pyhermes/base/sfc_projection.py:125-193: array input, or a
        catalogue file named by fin.path."""
        if self.particle_pos is None:
            p_pos, cw, fv = self._read_catalogue()
            n = p_pos.shape[0]
        else:
            p_pos = self.particle_pos
            if isinstance(p_pos, torch.Tensor):
                n = p_pos.shape[0]
            else:
                p_pos = np.asarray(p_pos)
                n = p_pos.shape[0]
            cw = self.catalog_weight
            fv = self.field_value
            self.fin["catalog_weight_key"] = None if cw is None else "custom"
            self.fin["field_value_key"] = None if fv is None else "custom"
        if p_pos.ndim != 2 or p_pos.shape[1] != 3:
            raise ValueError(
                "Wrong input of particle data! 'particle_pos' must be a 2D array of shape (N, 3), "
                f"but got shape={tuple(p_pos.shape)}."
            )
        self.particle_count = n
        if cw is None:
            cw = np.ones(n, dtype=np.float32)
        if fv is None:
            fv = np.ones(n, dtype=np.float32)
        factors = {}
        for name, value in (("catalog_weight", cw), ("field_value", fv)):
            if np.isscalar(value):
                value = np.full(n, value, dtype=np.float64)
            value = np.asarray(value)
            if value.ndim != 1 or value.shape[0] != n:
                raise ValueError(f"Wrong input of {name}! Expected shape ({n},), got {value.shape}.")
            if not np.all(np.isfinite(value)):
                raise ValueError(f"Wrong input of {name}! Values must all be finite.")
            factors[name] = value.astype(np.float64, copy=False)
        return p_pos, factors["catalog_weight"], factors["field_value"]

    def prepare_input_fields(self, particle_pos=None, catalog_weight=None, field_value=None, fin=None):
        if fin is not None:
            self.fin.update(fin)
        if particle_pos is not None:
            self.particle_pos = particle_pos
        if catalog_weight is not None:
            self.catalog_weight = catalog_weight
        if field_value is not None:
            self.field_value = field_value
        self.phi_array = sample_scaling_function(self.wavelet_mode, self.wavelet_level)
        self.phi_support = self.phi_array.shape[0] // self.phi_resolution
        self.scale_factor = self.L / self.box_size
        p_pos, cw, fv = self._load_particle_input()
        self.particle_pos = p_pos
        self.catalog_weight = cw
        self.field_value = fv
        # float64 normalisation, same expressions as the reference (:251-282)
        self.catalog_weight_sum = float(np.sum(cw, dtype=np.float64))
        self.catalog_weight_sq_sum = float(np.sum(cw ** 2, dtype=np.float64))
        if not np.isfinite(self.catalog_weight_sum) or np.isclose(self.catalog_weight_sum, 0.0):
            raise ValueError(f"Catalogue weights must have a finite, non-zero sum, got {self.catalog_weight_sum!r}.")
        self.raw_field_weighted_sum = float(np.sum(cw * fv, dtype=np.float64))
        if not np.isfinite(self.raw_field_weighted_sum):
            raise ValueError("The product catalog_weight * field_value produced a non-finite summed field value.")
        if self.weight_normalization == "raw":
            den = 1.0
        elif self.weight_normalization == "catalog":
            den = self.catalog_weight_sum
        else:
            den = self.raw_field_weighted_sum
            if np.isclose(den, 0.0):
                raise ValueError("weight_normalization='field' requires a finite, non-zero raw_field_weighted_sum.")
        self.projection_weight = cw * fv / den
        self.field_integral = self.raw_field_weighted_sum / den
        if self.save_particle_data:
            self._save_particle_dataset()
        self._fields_prepared = True

    def _save_particle_dataset(self):
        """pyhermes/base/sfc_projection.py:195-219: positions (float32),
        catalogue weights and field values (float64) as an npz at
        particle_data_path, or next to fout_path as <name>_particles.npz."""
        path = self.particle_data_path
        if not path:
            if not self.fout_path:
                raise ValueError("save_particle_data=True requires either 'particle_data_path' or 'fout_path' "
                                 "so the particle dataset has a place to go.")
            path = f"{os.path.splitext(self.fout_path)[0]}_particles.npz"
        d = os.path.dirname(path)
        if d:
            os.makedirs(d, exist_ok=True)
        pos = self.particle_pos.cpu().numpy() if isinstance(self.particle_pos, torch.Tensor) else self.particle_pos
        np.savez(path, pos=np.ascontiguousarray(pos, dtype=np.float32),
                 catalog_weight=np.ascontiguousarray(self.catalog_weight, dtype=np.float64),
                 field_value=np.ascontiguousarray(self.field_value, dtype=np.float64))
        self.particle_data_path = path

    def run(self, save_result=True, overwrite=False, out_dtype=torch.float32):
        t0 = time.perf_counter()
        if not self._fields_prepared:
            self.prepare_input_fields()
        dev = self.device
        pos = kernels.to_device(self.particle_pos, torch.float64, dev)
        w = kernels.to_device(self.projection_weight, torch.float64, dev)
        phi = kernels.to_device(self.phi_array, torch.float64, dev)
        eps, _, ws = kernels.deposit(pos, w, self.J, float(self.box_size), phi, self.phi_resolution,
                                     out_dtype=out_dtype, workspace=self._workspace)
        rejected = kernels.deposit_rejected(ws, dev)
        if rejected:
            raise ValueError(f"{rejected} particles have non-finite or out-of-range positions.")
        field = SFCField(threads=self.threads, device=dev)
        field.sfc_info = {
            "fin": copy.deepcopy(self.fin),
            "particle_count": self.particle_count,
            "catalog_weight_sum": self.catalog_weight_sum,
            "catalog_weight_sq_sum": self.catalog_weight_sq_sum,
            "raw_field_weighted_sum": self.raw_field_weighted_sum,
            "field_integral": self.field_integral,
            "box_size": self.box_size,
            "J": self.J,
            "L": self.L,
            "V": self.L ** 3,
            "scale_factor": self.scale_factor,
            "field_kind": "catalog_field",
            "weight_normalization": self.weight_normalization,
            "particle_data_retrievable": True,
            "wavelet_mode": self.wavelet_mode,
            "wavelet_level": self.wavelet_level,
            "phi_resolution": self.phi_resolution,
            "particle_data_path": self.particle_data_path if self.save_particle_data else "",
            "particle_data_format": "npz" if self.save_particle_data else "",
            "phi_support": self.phi_support,
            "phi_array": self.phi_array,
        }
        field.format_sfc_params()
        field.epsilon_device = eps
        self.sfc_field = field
        if save_result and self.fout_path:
            field.save_sfc_field(self.fout_path, overwrite=overwrite)
        logger.info("SFCProjection J=%d n=%d in %.4f s", self.J, self.particle_count, time.perf_counter() - t0)
        return field
