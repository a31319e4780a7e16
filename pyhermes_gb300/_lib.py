"""ctypes binding of ``libhermes_gb300.so`` (the C ABI in include/hermes_gb300.h).

The library is required: there is no CPU fallback.  If it is missing the
first call raises ``HermesLibraryError`` telling the user to build it.
"""

import ctypes
import os
import re

from .build import LIB_PATH, PKG_DIR

HEADER_PATH = os.path.join(PKG_DIR, "..", "include", "hermes_gb300.h")

_c_int = ctypes.c_int
_c_i64 = ctypes.c_int64
_c_sz = ctypes.c_size_t
_p = ctypes.c_void_p
_dbl = ctypes.c_double

# name -> (restype, argtypes)
SIGNATURES = {
    "hermes_version": (ctypes.c_char_p, []),
    "hermes_last_error": (ctypes.c_char_p, []),
    "hermes_deposit_workspace_size": (_c_int, [_c_i64, _c_int, ctypes.POINTER(_c_sz)]),
    "hermes_deposit": (_c_int, [_p, _p, _c_i64, _c_int, _dbl, _p, _c_int, _c_int,
                                _p, _p, _p, _p, _c_sz, _p]),
    "hermes_deposit_sort": (_c_int, [_p, _p, _c_i64, _c_int, _dbl, _p, _c_int, _c_int, _p, _c_sz, _p]),
    "hermes_deposit_accumulate": (_c_int, [_c_i64, _c_int, _dbl, _p, _c_int, _c_int, _p, _p, _p,
                                           _p, _c_sz, _p]),
    "hermes_deposit_status": (_c_int, [_p, ctypes.POINTER(_c_i64), _p]),
    "hermes_deposit_set_tile": (_c_int, [_c_int, _c_int, _c_int, _c_int]),
    "hermes_phi_prepare": (_c_int, [_p, _c_int, _c_int, _c_int, _c_int, _p, _p, _p]),
    "hermes_deposit_get_tile": (_c_int, [_c_int, ctypes.POINTER(_c_int), ctypes.POINTER(_c_int),
                                         ctypes.POINTER(_c_int)]),
    "hermes_deposit_noalloc": (_c_int, [_p, _p, _c_i64, _c_int, _dbl, _p, _c_int, _c_int, _p, _p, _p, _p]),
    "hermes_fft_r2c": (_c_int, [_p, _p, _c_int, _p]),
    "hermes_fft_c2r": (_c_int, [_p, _p, _c_int, _p]),
    "hermes_window_workspace_size": (_c_int, [_c_int, ctypes.POINTER(_c_sz)]),
    "hermes_window_apply": (_c_int, [_p, _p, _c_int, _p, _p, _c_int, _p, _c_sz, _p]),
    "hermes_window_materialize": (_c_int, [_p, _p, _c_int, _c_int, _p, _p, _p]),
    "hermes_spectrum_multiply": (_c_int, [_p, _p, _p, _c_int, _dbl, _p]),
    "hermes_pair_products_workspace_size": (_c_int, [_c_int, _c_int, _c_int, ctypes.POINTER(_c_sz)]),
    "hermes_pair_products": (_c_int, [_p, _c_int, _p, _c_int, _p, _c_int, _p, _c_int, _c_int, _c_int,
                                      _p, _p, _p, _c_sz, _p]),
    "hermes_multipole_workspace_size": (_c_int, [_c_int, _c_int, ctypes.POINTER(_c_sz)]),
    "hermes_multipole_fields": (_c_int, [_p, _c_int, _c_int, _c_int, _p, _c_int, _p, _p, _p, _c_sz, _p]),
    "hermes_multipole_contract": (_c_int, [_p, _p, _c_int, _p, _c_int, _c_int, _p, _c_int, _p, _p, _c_sz, _p]),
    "hermes_multipole_fields_window": (_c_int, [_p, _c_int, _c_int, _c_int, _p, _c_int, _p, _p, _p, _c_sz, _p]),
    "hermes_multipole_fields_table": (_c_int, [_p, _c_int, _c_int, _c_int, _p, _p, _p, _p, _dbl, _c_int, _p, _p, _p,
                                               _c_sz, _p]),
    "hermes_multipole_contract_async": (_c_int, [_p, _p, _c_int, _p, _c_int, _c_int, _p, _c_int, _c_int, _c_int, _p, _p,
                                                 _c_sz, _p]),
    "hermes_multipole_contract_simt_async": (_c_int, [_p, _p, _c_int, _p, _c_int, _c_int, _p, _c_int, _c_int, _c_int,
                                                      _p, _p, _c_sz, _p]),
    "hermes_multipole_fields_bm": (_c_int, [_p, _c_int, _c_int, _c_int, _p, _c_int, _p, _p, _p, _c_sz, _p]),
    "hermes_multipole_fields_window_bm": (_c_int, [_p, _c_int, _c_int, _c_int, _p, _c_int, _p, _p, _p, _c_sz, _p]),
    "hermes_multipole_fields_table_bm": (_c_int, [_p, _c_int, _c_int, _c_int, _p, _p, _p, _p, _dbl, _c_int, _p, _p,
                                                  _p, _c_sz, _p]),
    "hermes_multipole_contract_bm_async": (_c_int, [_p, _p, _c_int, _p, _c_int, _c_int, _p, _c_int, _c_int, _c_int,
                                                    _p, _p, _c_sz, _p]),
    "hermes_multipole_set_fft": (_c_int, [_c_int]),
    "hermes_fft512_strided_inverse": (_c_int, [_p, _c_int, _c_int, _p]),
    "hermes_multipole_fields_pair_bm": (_c_int, [_p, _c_int, _c_int, _p, _c_int, _p, _p, _p, _c_sz, _p]),
    "hermes_multipole_contract_pair_bm_async": (_c_int, [_p, _p, _c_int, _p, _c_int, _c_int, _c_int, _p, _p, _c_sz,
                                                         _p]),
    "hermes_multipole_contract_status": (_c_int, [_p, _c_sz, _c_int, ctypes.POINTER(_c_int), _p]),
    "hermes_multipole_contract_plain": (_c_int, [_p, _p, _p, _p, _c_int, _p, _p, _c_sz, _p]),
    "hermes_mixing_solve": (_c_int, [_p, _p, _p, _c_int, _c_int, _p, _p, _p, _p]),
    "hermes_mc_workspace_size": (_c_int, [ctypes.POINTER(_c_sz)]),
    "hermes_mc_sample": (_c_int, [_p, _p, _p, _c_int, _p, ctypes.c_int64, _p, _p, _p, ctypes.c_int64, ctypes.c_double,
                                  ctypes.c_double, ctypes.c_double, ctypes.c_uint64, _p, _c_int, _c_int, _p, _p, _c_sz,
                                  _p]),
    "hermes_interp": (_c_int, [_p, _c_int, _p, _c_i64, _p, _c_int, _c_int, _dbl, _dbl, _dbl, _p, _p, _c_sz, _p]),
    "hermes_mc_triplets": (_c_int, [_p, _p, _p, _c_int, _p, _p, _c_i64, _p, _c_int, _p, _c_int, _c_int, _dbl,
                                    ctypes.POINTER(_dbl), _p, _p, _c_sz, _p]),
    "hermes_mc_triplets_bricks": (_c_int, [_p, _p, _p, _c_int, _p, _p, _c_i64, _p, _c_int, _p, _c_int, _c_int, _dbl,
                                           ctypes.POINTER(_dbl), _p, _p, _c_sz, _p]),
    "hermes_mc_sample_bricks": (_c_int, [_p, _p, _p, _c_int, _p, ctypes.c_int64, _p, _p, _p, ctypes.c_int64,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_uint64, _p,
                                         _c_int, _c_int, _p, _p, _c_sz, _p]),
    "hermes_field_to_bricks": (_c_int, [_p, _c_int, _p, _p]),
    "hermes_mlp_infer_tc": (_c_int, [_p, _p, _c_int, _p, _c_i64, _p, _p, _p]),
    "hermes_poisson_grad": (_c_int, [_p, _p, _c_i64, _p, ctypes.POINTER(_dbl), _p, _p]),
    "hermes_mlp_param_count": (_c_int, [_p, _c_int, ctypes.POINTER(_c_i64)]),
    "hermes_mlp_scratch_floats": (_c_int, [_c_i64, ctypes.POINTER(_c_i64)]),
    "hermes_mlp_forward": (_c_int, [_p, _p, _p, _c_int, _p, _c_i64, _p, _p]),
    "hermes_mlp_backward": (_c_int, [_p, _p, _c_int, _p, _c_i64, _p, _p, _p, _p, _p]),
    "hermes_mse_grad": (_c_int, [_p, _p, _c_i64, _p, ctypes.POINTER(_dbl), _p, _p]),
    "hermes_adam_step": (_c_int, [_p, _p, _p, _p, _c_i64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                  ctypes.c_float, _c_int, _p]),
    "hermes_to_bf16": (_c_int, [_p, _c_i64, _p, _p]),
}


class HermesLibraryError(RuntimeError):
    """The CUDA library is missing or could not be loaded."""


class HermesError(RuntimeError):
    """A hermes_* call returned a non-zero status."""

    def __init__(self, code, message):
        super().__init__(f"hermes error {code}: {message}")
        self.code = code


_LIB = None


def header_symbols():
    """Every function name declared in include/hermes_gb300.h."""
    text = open(HEADER_PATH).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hermes_[a-z0-9_]+)\s*\(", text)))


def load():
    """Load (once) and return the library with argument types declared."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise HermesLibraryError(
            f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
            "or `python -m pyhermes_gb300.build`."
        )
    try:
        lib = ctypes.CDLL(LIB_PATH)
    except OSError as exc:
        raise HermesLibraryError(f"cannot load {LIB_PATH}: {exc}") from exc
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(rc, what=""):
    if rc != 0:
        msg = load().hermes_last_error().decode(errors="replace")
        raise HermesError(rc, f"{what}: {msg}" if what else msg)
