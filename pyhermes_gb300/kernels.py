"""Thin torch-facing wrappers over the C ABI.

Each wrapper validates shapes on the host, allocates outputs and workspaces
as torch CUDA tensors, and launches on torch's current stream.  All compute
happens in ``libhermes_gb300.so``; there is no CPU fallback.
"""

import ctypes

import numpy as np
import torch

from . import _lib


def _stream_ptr(device=None):
    return torch.cuda.current_stream(device).cuda_stream


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def require_cuda(t, name, dtype=None):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


def to_device(a, dtype, device="cuda"):
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=device)


class DepositWorkspace:
    """Reusable scratch for hermes_deposit (grows on demand)."""

    def __init__(self, device="cuda"):
        self.device = device
        self.buf = None

    def get(self, n, J):
        need = ctypes.c_size_t(0)
        _lib.check(_lib.load().hermes_deposit_workspace_size(int(n), int(J), ctypes.byref(need)),
                   "hermes_deposit_workspace_size")
        if self.buf is None or self.buf.numel() < need.value:
            self.buf = torch.empty(max(int(need.value), 256), dtype=torch.uint8, device=self.device)
        return self.buf


def deposit(pos, w, J, box, phi, phi_res=1024, out_dtype=torch.float32, counts=False,
            workspace=None, out=None):
    """Scaling-function deposit on the GPU.

    pos: (n,3) float64 CUDA tensor; w: (n,) float64; phi: (n_phi,) float64.
    Returns (eps[L,L,L] of ``out_dtype``, counts[L,L,L] uint32 or None, workspace).
    """
    require_cuda(pos, "pos", torch.float64)
    require_cuda(w, "w", torch.float64)
    require_cuda(phi, "phi", torch.float64)
    if pos.ndim != 2 or pos.shape[1] != 3:
        raise ValueError(f"pos must have shape (n, 3), got {tuple(pos.shape)}")
    n = pos.shape[0]
    if w.shape != (n,):
        raise ValueError(f"w must have shape ({n},), got {tuple(w.shape)}")
    L = 1 << int(J)
    dev = pos.device
    if out is None:
        out = torch.empty((L, L, L), dtype=out_dtype, device=dev)
    cnt = torch.empty((L, L, L), dtype=torch.int32, device=dev) if counts else None
    ws = workspace if workspace is not None else DepositWorkspace(dev)
    buf = ws.get(n, J)
    lib = _lib.load()
    e32 = out if out.dtype == torch.float32 else None
    e64 = out if out.dtype == torch.float64 else None
    if e32 is None and e64 is None:
        raise TypeError("out_dtype must be float32 or float64")
    rc = lib.hermes_deposit(_ptr(pos), _ptr(w), n, int(J), float(box), _ptr(phi), phi.numel(),
                            int(phi_res), _ptr(e32), _ptr(e64), _ptr(cnt), _ptr(buf),
                            buf.numel(), _stream_ptr(dev))
    _lib.check(rc, "hermes_deposit")
    return out, cnt, ws


def deposit_rejected(ws, device=None):
    """Number of particles the last deposit skipped (non-finite / out of range)."""
    n = ctypes.c_int64(0)
    _lib.check(_lib.load().hermes_deposit_status(_ptr(ws.buf), ctypes.byref(n), _stream_ptr(device)),
               "hermes_deposit_status")
    return int(n.value)
