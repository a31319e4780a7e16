"""Tile autotuner for the multipole contraction.

``tune_contract(J, nb)`` times ``hermes_multipole_contract_bm_async`` on the
current GPU for each x-chunk length (planes per work item: the halo of 4
planes costs 4/CX, a short chunk gives more work items for load balance)
and 1 or 2 CTAs per SM, with CUDA events after a warm-up, and returns the
fastest choice.  Results are cached per (device, J, nb) for the process.
The deposit tiles (8 x 16 x 32 cells) are fixed at compile time.
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
