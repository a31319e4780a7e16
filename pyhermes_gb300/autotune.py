"""Tile autotuners for the multipole contraction and the deposit.

``tune_contract(J, nb)`` times ``hermes_multipole_contract_bm_async`` on the
current GPU for each x-chunk length (planes per work item: the halo of 4
planes costs 4/CX, a short chunk gives more work items for load balance)
and 1 or 2 CTAs per SM, with CUDA events after a warm-up, and returns the
fastest choice.  Results are cached per (device, J, nb) for the process.

``tune_deposit(pos, w, J, box, phi)`` times the deposit (sort + tile
accumulation) of the caller's own catalogue for each candidate tile shape
(``DEPOSIT_TILES``, clipped to the grid), keeps the fastest for level J
(``hermes_deposit_set_tile``) and returns it.  Every tile gives the same
field bit for bit (integer fixed-point sums), which the tuner checks.
Results are cached per (device, J, log2 n) for the process.
"""

import ctypes

import numpy as np
import torch

from . import multipole as mp

_CACHE = {}
CHUNKS = (16, 32, 64, 128)
CTAS = (1, 2)


def tune_contract(J, nb, device="cuda", reps=3):
    """(chunk_x, ctas_per_sm, timings) for a J, nb-radius contraction."""
    dev = torch.device(device)
    key = (torch.cuda.get_device_name(dev), int(J), int(nb))
    if key in _CACHE:
        return _CACHE[key]
    L = 1 << J
    g = torch.Generator(device=dev).manual_seed(1)
    eps = torch.randn((L, L, L), generator=g, device=dev, dtype=torch.float32)
    # bin-major fields [nb, L^3], the layout the tensor-core engine reads
    fields = torch.view_as_complex(torch.randn((nb, L ** 3, 2), generator=g, device=dev, dtype=torch.float32))
    out = torch.zeros((mp.MAX_BINS, mp.MAX_BINS, 2), dtype=torch.float64, device=dev)
    gamma = (ctypes.c_double * 9)(*np.full(9, 1.0 / 9.0))
    stream = torch.cuda.current_stream(dev)
    timings = {}
    for cx in CHUNKS:
        if cx > L:
            continue
        for ctas in CTAS:
            for _ in range(2):
                mp.multipole_contract_async(eps, fields, nb, gamma, J, out, conj_sign=1, chunk_x=cx, ctas_per_sm=ctas,
                                            bin_major=True)
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
            for a, b in ev:
                a.record(stream)
                mp.multipole_contract_async(eps, fields, nb, gamma, J, out, conj_sign=1, chunk_x=cx, ctas_per_sm=ctas,
                                            bin_major=True)
                b.record(stream)
            torch.cuda.synchronize(dev)
            timings[(cx, ctas)] = min(a.elapsed_time(b) for a, b in ev)
    best = min(timings, key=timings.get)
    _CACHE[key] = (best[0], best[1], {f"cx{k[0]}_ctas{k[1]}": v for k, v in timings.items()})
    return _CACHE[key]


DEPOSIT_TILES = ((8, 16, 32), (8, 8, 32), (4, 16, 32), (16, 16, 32), (8, 32, 32), (16, 16, 16), (8, 16, 64),
                 (16, 32, 32), (4, 32, 64))
_DEP_CACHE = {}


def deposit_tile(J):
    """The tile shape (x, y, z) the deposit uses at level J."""
    from . import _lib

    t = [ctypes.c_int(0) for _ in range(3)]
    _lib.check(_lib.load().hermes_deposit_get_tile(int(J), *[ctypes.byref(v) for v in t]), "hermes_deposit_get_tile")
    return tuple(v.value for v in t)


def set_deposit_tile(J, tile):
    """Sets the deposit tile of level J ((0, 0, 0): the default)."""
    from . import _lib

    _lib.check(_lib.load().hermes_deposit_set_tile(int(J), *[int(v) for v in tile]), "hermes_deposit_set_tile")


def tune_deposit(pos, w, J, box, phi, reps=3):
    """Fastest tile shape for depositing this catalogue at level J; sets it
    for J and returns (tile, {tile: ms}).  pos, w, phi: float64 CUDA tensors
    as for kernels.deposit."""
    import math

    from . import kernels

    dev = pos.device
    n = int(pos.shape[0])
    key = (torch.cuda.get_device_name(dev), int(J), int(math.log2(max(n, 1))))
    if key in _DEP_CACHE:
        set_deposit_tile(J, _DEP_CACHE[key][0])
        return _DEP_CACHE[key]
    L = 1 << int(J)
    stream = torch.cuda.current_stream(dev)
    ws = kernels.DepositWorkspace(dev)
    out = torch.empty((L, L, L), dtype=torch.float32, device=dev)
    ref = None
    timings = {}
    seen = set()
    for cand in DEPOSIT_TILES:
        clipped = tuple(min(c, L) for c in cand)
        if clipped in seen:
            continue
        seen.add(clipped)
        set_deposit_tile(J, cand)
        kernels.deposit(pos, w, J, box, phi, workspace=ws, out=out)
        if ref is None:
            ref = out.clone()
        elif not torch.equal(out, ref):
            set_deposit_tile(J, (0, 0, 0))
            raise RuntimeError(f"deposit tile {cand} changed the field")
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, b in ev:
            a.record(stream)
            kernels.deposit(pos, w, J, box, phi, workspace=ws, out=out)
            b.record(stream)
        torch.cuda.synchronize(dev)
        timings[cand] = min(a.elapsed_time(b) for a, b in ev)
    best = min(timings, key=timings.get)
    set_deposit_tile(J, best)
    _DEP_CACHE[key] = (best, {"x".join(map(str, k)): v for k, v in timings.items()})
    return _DEP_CACHE[key]
