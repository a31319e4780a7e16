"""The reference's data-container import path (pyhermes/io/__init__.py):
fields, windows, result containers, the NumPy-framed pickle and the output
path rules."""
from ..corr2pcf import Corr2PCFData
from ..counting import CountingData
from ..mc3pcf import Corr3PCFData
from ..multipole import Corr3PCFMultipoleData
from ..sfc_field import (SFCField, check_fout, normalize_task_weight_normalization, normalize_weight_normalization,
                         read_numpy_pickle, write_numpy_pickle)
from ..window import WindowFunc

__all__ = ["SFCField", "WindowFunc", "Corr2PCFData", "Corr3PCFData", "Corr3PCFMultipoleData", "CountingData",
           "normalize_task_weight_normalization", "normalize_weight_normalization", "check_fout",
           "read_numpy_pickle", "write_numpy_pickle"]
