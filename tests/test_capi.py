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


def test_deposit_tile_setting(lib):
    """The per-level deposit tile: validated, read back (clipped to the grid),
    reflected in the workspace size, and reset to the default."""
    t = [ctypes.c_int(0) for _ in range(3)]
    refs = [ctypes.byref(v) for v in t]
    assert lib.hermes_deposit_get_tile(7, *refs) == 0
    assert [v.value for v in t] == [8, 16, 32]
    base = ctypes.c_size_t(0)
    assert lib.hermes_deposit_workspace_size(100000, 7, ctypes.byref(base)) == 0
    try:
        assert lib.hermes_deposit_set_tile(7, 4, 8, 16) == 0
        assert lib.hermes_deposit_get_tile(7, *refs) == 0
        assert [v.value for v in t] == [4, 8, 16]
        small = ctypes.c_size_t(0)
        assert lib.hermes_deposit_workspace_size(100000, 7, ctypes.byref(small)) == 0
        assert small.value > base.value  # more tiles, more bucket counters
        assert lib.hermes_deposit_set_tile(3, 16, 16, 32) == 0  # clipped to L = 8 on read
        assert lib.hermes_deposit_get_tile(3, *refs) == 0
        assert [v.value for v in t] == [8, 8, 8]
        for bad in [(7, 3, 16, 32), (7, 2, 16, 32), (7, 8, 16, 2), (7, 256, 16, 32), (7, 32, 32, 32),
                    (11, 8, 16, 32), (1, 8, 16, 32)]:
            assert lib.hermes_deposit_set_tile(*bad) == -1, bad
            assert b"deposit_set_tile" in lib.hermes_last_error()
    finally:
        assert lib.hermes_deposit_set_tile(7, 0, 0, 0) == 0
        assert lib.hermes_deposit_set_tile(3, 0, 0, 0) == 0
    again = ctypes.c_size_t(0)
    assert lib.hermes_deposit_workspace_size(100000, 7, ctypes.byref(again)) == 0
    assert again.value == base.value


def test_phi_prepare_rejects_bad_arguments(lib):
    assert lib.hermes_phi_prepare(None, 3072, 1024, 64, 1, None, None, None) == -1
    assert b"phi is NULL" in lib.hermes_last_error()


def test_degree_pair_entries_reject_bad_arguments(lib):
    # odd or out-of-range degrees are refused before any device work
    for l in (1, 3, -2, 40):
        assert lib.hermes_multipole_fields_pair_bm(None, 7, l, None, 4, None, None, None, 0, None) == -1, l
        assert b"multipole_fields_pair" in lib.hermes_last_error()
    assert lib.hermes_multipole_contract_pair_bm_async(None, None, 4, None, 7, 0, 0, None, None, 0, None) == -1


def test_fft_mode_switch(lib):
    prev = lib.hermes_multipole_set_fft(0)
    assert prev in (0, 1)
    assert lib.hermes_multipole_set_fft(prev) == 0
    for bad in (-1, 2):
        assert lib.hermes_multipole_set_fft(bad) == -1
        assert b"multipole_set_fft" in lib.hermes_last_error()
    assert lib.hermes_fft512_strided_inverse(None, 1, 0, None) == -1
