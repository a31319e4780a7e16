"""The C-ABI library builds for sm_103a, loads, and exports every symbol the
public header declares (no GPU needed)."""
import ctypes

import pytest

from pyhermes_gb300 import _lib, build


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_exports_every_header_symbol(lib):
    names = _lib.header_symbols()
    assert "hermes_deposit" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"symbols declared in include/hermes_gb300.h but not exported: {missing}"


def test_every_header_symbol_has_a_binding():
    names = _lib.header_symbols()
    assert sorted(n for n in names if n not in _lib.SIGNATURES) == []


def test_version_and_error_paths(lib):
    assert b"sm_103a" in lib.hermes_version()
    size = ctypes.c_size_t(0)
    assert lib.hermes_deposit_workspace_size(1000, 7, ctypes.byref(size)) == 0
    assert size.value > 1000 * 32
    # invalid J is rejected with a message, without touching the GPU
    rc = lib.hermes_deposit_workspace_size(1000, 15, ctypes.byref(size))
    assert rc == -1
    assert b"J=15" in lib.hermes_last_error()
    assert lib.hermes_deposit_workspace_size(1000, 7, None) == -1
