"""The reference's data-container import path (pyhermes/io/__init__.py):
fields, windows, result containers, the NumPy-framed pickle, the output
path rules and the catalogue readers."""
from ..corr2pcf import Corr2PCFData
from ..counting import CountingData
from ..mc3pcf import Corr3PCFData
from ..multipole import Corr3PCFMultipoleData
from ..readers import (FORMAT_READERS, infer_format, read_bin, read_fof, read_gadget, read_gadget_fof,
                       read_gadget_hdf5, read_npz, read_particle_data, resolve_particle_value)
from ..resources import file_sha256, is_remote_url, remote_cache_path, resolve_data_path
from ..sfc_field import (SFCField, check_fout, normalize_task_weight_normalization, normalize_weight_normalization,
                         read_numpy_pickle, write_numpy_pickle)
from ..window import WindowFunc

__all__ = ["SFCField", "WindowFunc", "Corr2PCFData", "Corr3PCFData", "Corr3PCFMultipoleData", "CountingData",
           "normalize_task_weight_normalization", "normalize_weight_normalization", "check_fout",
           "read_numpy_pickle", "write_numpy_pickle", "FORMAT_READERS", "infer_format", "read_bin", "read_npz",
           "read_gadget", "read_gadget_hdf5", "read_gadget_fof", "read_fof", "read_particle_data",
           "resolve_particle_value", "file_sha256", "is_remote_url", "remote_cache_path", "resolve_data_path"]
