"""hermes_deposit_noalloc: the deposit for callers that cannot allocate
device memory, whose scratch is an array built into the library.

Called through the C ABI twice in a row (different catalogues, so stale
scratch from the first call would show) and compared with hermes_deposit
(caller workspace) within the deposit tolerance used elsewhere in the suite
(2e-6 of max|eps|; the fixed-point accumulation in fact makes them equal).
Collected last so a failure here leaves the rest of the suite already run.
"""
import ctypes

import numpy as np
import pytest
import torch

from pyhermes_gb300 import _lib, kernels
from pyhermes_gb300.phi import sample_scaling_function

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _catalogue(seed, n):
    rng = np.random.default_rng(seed)
    pos = torch.as_tensor(rng.uniform(0.0, 1000.0, (n, 3)), device="cuda")
    w = torch.as_tensor(rng.lognormal(0.0, 0.3, n) / n, device="cuda")
    return pos, w


def test_noalloc_deposit_matches_workspace_deposit_twice():
    lib = _lib.load()
    phi = torch.as_tensor(sample_scaling_function(), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for seed, n, J in ((1, 100_000, 7), (2, 131_072, 8)):
        pos, w = _catalogue(seed, n)
        L = 1 << J
        eps = torch.empty((L, L, L), dtype=torch.float32, device="cuda")
        cnt = torch.empty((L, L, L), dtype=torch.int32, device="cuda")
        rc = lib.hermes_deposit_noalloc(_ptr(pos), _ptr(w), n, J, 1000.0, _ptr(phi), phi.numel(), 1024,
                                        _ptr(eps), None, _ptr(cnt), stream)
        _lib.check(rc, "hermes_deposit_noalloc")
        ref, ref_cnt, _ = kernels.deposit(pos, w, J, 1000.0, phi, counts=True)
        torch.cuda.synchronize()
        scale = ref.abs().max().item()
        assert (eps - ref).abs().max().item() <= 2e-6 * scale
        assert torch.equal(eps, ref)
        assert torch.equal(cnt, ref_cnt)


def test_noalloc_deposit_rejects_sizes_beyond_its_scratch():
    lib = _lib.load()
    phi = torch.as_tensor(sample_scaling_function(), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    pos, w = _catalogue(3, 16)
    eps = torch.empty((8, 8, 8), dtype=torch.float32, device="cuda")
    rc = lib.hermes_deposit_noalloc(_ptr(pos), _ptr(w), 16, 9, 1000.0, _ptr(phi), phi.numel(), 1024, _ptr(eps),
                                    None, None, stream)
    assert rc == -1 and b"J=9" in lib.hermes_last_error()
    rc = lib.hermes_deposit_noalloc(_ptr(pos), _ptr(w), 131_073, 5, 1000.0, _ptr(phi), phi.numel(), 1024,
                                    _ptr(eps), None, None, stream)
    assert rc == -1 and b"n=131073" in lib.hermes_last_error()


def test_noalloc_deposit_float64_output_and_output_choice():
    """The float64 field output on the built-in scratch equals
    kernels.deposit(..., out_dtype=float64) bit for bit, and giving both
    outputs or neither is refused."""
    lib = _lib.load()
    phi = torch.as_tensor(sample_scaling_function(), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    n, J = 50_000, 6
    pos, w = _catalogue(4, n)
    L = 1 << J
    e64 = torch.empty((L, L, L), dtype=torch.float64, device="cuda")
    rc = lib.hermes_deposit_noalloc(_ptr(pos), _ptr(w), n, J, 1000.0, _ptr(phi), phi.numel(), 1024, None, _ptr(e64),
                                    None, stream)
    _lib.check(rc, "hermes_deposit_noalloc")
    ref, _, _ = kernels.deposit(pos, w, J, 1000.0, phi, out_dtype=torch.float64)
    torch.cuda.synchronize()
    assert torch.equal(e64, ref)
    e32 = torch.empty((L, L, L), dtype=torch.float32, device="cuda")
    rc = lib.hermes_deposit_noalloc(_ptr(pos), _ptr(w), n, J, 1000.0, _ptr(phi), phi.numel(), 1024, _ptr(e32),
                                    _ptr(e64), None, stream)
    assert rc == -1
    rc = lib.hermes_deposit_noalloc(_ptr(pos), _ptr(w), n, J, 1000.0, _ptr(phi), phi.numel(), 1024, None, None,
                                    None, stream)
    assert rc == -1
