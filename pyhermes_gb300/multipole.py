"""3PCF spherical-harmonic multipoles on the GPU.

``Corr_3PCF_Multipole`` mirrors ``pyhermes/theory/corr3pcf_multipole.py``
(serial semantics): the same parameter dict (sampling in grid / paired mode,
binning_window12/13 with a mapping from sampled names to ``len_args``),
products ddd_l / rrr_l / delta_ddd_l / zeta_l, the all-uniform analytic
rrr_l shortcut (:1389-1395), the physical rescale by scale_factor**9
(:546-555, :944-952) and the zeta_l mixing-matrix solve (:1554-1589,
utils/special_functions.py:337-409).

Engine (``MultipoleEngine``): instead of rebuilding both side fields for
every (r12, r13) sample as the reference does (calc_DDD_multipole per
sample), each (l, m) produces the a_lm fields of every distinct radius once
(``hermes_multipole_fields``) and contracts all radius pairs at once
(``hermes_multipole_contract``).  When the second and third vertices share
the field and the radii, a_{l,-m} = (-1)^{l+m} conj(a_lm) removes the
second batch.  ``summation_backend='plain'`` runs the per-sample reference
form on the GPU (the baseline the batched engine is measured against).
"""

import copy
import ctypes
import itertools
import math
import logging
import time

import numpy as np
import torch

from . import _lib
from .kernels import _ptr, _stream_ptr
from .params import task_params
from .phi import cal_gamma, sample_scaling_function
from .sfc_field import (ResultFileIO, SFCField, check_fout, describe_input, normalize_task_weight_normalization,
                        read_numpy_pickle, write_numpy_pickle)
from .window import WindowFunc, phi_power_device, rfft_field

logger = logging.getLogger("pyhermes_gb300.Corr_3PCF_Multipole")

MAX_BINS = 16
_WS = {}


def _workspace(nbytes, device):
    device = torch.device(device)
    if device.type == "cuda" and device.index is None:
        device = torch.device("cuda", torch.cuda.current_device())
    key = ("multipole", str(device))
    buf = _WS.get(key)
    if buf is None or buf.numel() < nbytes:
        if buf is not None:
            del _WS[key]
            buf = None
            torch.cuda.empty_cache()
        buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
        _WS[key] = buf
    return buf


def _ws_bytes(J, nb):
    n = ctypes.c_size_t(0)
    _lib.check(_lib.load().hermes_multipole_workspace_size(J, nb, ctypes.byref(n)), "multipole_workspace_size")
    return n.value


BIN_STRIDE = 16


def _fields_out(J, nb, bin_major, dev):
    N = 1 << (3 * J)
    shape = (N,) if nb == 1 else ((nb, N) if bin_major else (N, BIN_STRIDE))
    return torch.empty(shape, dtype=torch.complex64, device=dev)


def fields_ws_bytes(J, nb, bin_major=False):
    """Workspace bytes of the fields calls: the bin-major layout needs no
    bin-major staging copy."""
    return _ws_bytes(J, 1 if bin_major else nb)


def multipole_fields(half_spec, J, l, m, radii_grid, phi_power, out=None, ws=None, bin_major=False):
    """a_lm^b = ifftn(fftn(eps) K_lm^b) for thin-shell radii (grid units).

    Returns complex64 [L^3, 16] (bin-interleaved; bins >= nb unused) for
    several radii, or [L^3] for a single radius.  bin_major=True returns
    [nb, L^3] as the inverse FFT leaves it (hermes_multipole_fields_bm: no
    interleave pass, no bin-major workspace copy), the layout the tensor-core
    contraction reads with bin_major=True."""
    nb = len(radii_grid)
    dev = half_spec.device
    if out is None:
        out = _fields_out(J, nb, bin_major, dev)
    if ws is None:
        ws = _workspace(fields_ws_bytes(J, nb, bin_major), dev)
    radii = (ctypes.c_double * nb)(*[float(r) for r in radii_grid])
    lib = _lib.load()
    fn = lib.hermes_multipole_fields_bm if bin_major else lib.hermes_multipole_fields
    _lib.check(fn(_ptr(half_spec), J, int(l), int(m), radii, nb, _ptr(phi_power), _ptr(out), _ptr(ws), ws.numel(),
                  _stream_ptr(dev)), "hermes_multipole_fields")
    return out


def multipole_fields_pair(half_spec, J, l, radii_grid, phi_power, out=None, ws=None):
    """a_{l,0} + a_{l+1,0} for even l and thin-shell radii (grid units),
    bin-major complex64 [nb, L^3] (hermes_multipole_fields_pair_bm): the real
    field a_{l,0} in the real part and the imaginary field a_{l+1,0} in the
    imaginary part, from one prepass and one inverse FFT."""
    nb = len(radii_grid)
    dev = half_spec.device
    if out is None:
        out = torch.empty((nb, 1 << (3 * J)), dtype=torch.complex64, device=dev)
    if ws is None:
        ws = _workspace(fields_ws_bytes(J, nb, True), dev)
    radii = (ctypes.c_double * nb)(*[float(r) for r in radii_grid])
    _lib.check(_lib.load().hermes_multipole_fields_pair_bm(_ptr(half_spec), J, int(l), radii, nb, _ptr(phi_power),
                                                           _ptr(out), _ptr(ws), ws.numel(), _stream_ptr(dev)),
               "hermes_multipole_fields_pair_bm")
    return out


def multipole_contract_pair_async(eps1, fields, nb, gamma_c, J, dev_out, chunk_x=0, ctas_per_sm=0, ws=None):
    """hermes_multipole_contract_pair_bm_async: dev_out[b2, b3] = (S_{l,0},
    S_{l+1,0}) (times 4 pi / L^3) from the fields of multipole_fields_pair."""
    dev = eps1.device
    if ws is None:
        ws = _workspace(_ws_bytes(J, 1), dev)
    _lib.check(_lib.load().hermes_multipole_contract_pair_bm_async(_ptr(eps1), _ptr(fields), nb, gamma_c, J,
                                                                   int(chunk_x), int(ctas_per_sm), _ptr(dev_out),
                                                                   _ptr(ws), ws.numel(), _stream_ptr(dev)),
               "hermes_multipole_contract_pair_bm_async")
    return dev_out


def degree_pairs(lms):
    """Even l with (l, 0) and (l + 1, 0) both in lms: the m = 0 terms one
    paired fields pass and contraction serve (a_{l,0} is real for even l and
    imaginary for odd l, so one complex field carries both)."""
    have = set(lms)
    return [l for l in sorted({l for l, _ in lms}) if l % 2 == 0 and (l, 0) in have and (l + 1, 0) in have]


class BinSpec:
    """One radial bin of a multipole window: radial profile type, physical
    len_args and the binning window's other_args (profile configuration)."""

    __slots__ = ("type", "len_args", "profile")

    def __init__(self, radial_type, len_args, profile=None):
        self.type = str(radial_type).strip().lower()
        self.len_args = {k: float(v) for k, v in dict(len_args).items()}
        self.profile = profile if profile else None

    def key(self):
        return (self.type, tuple(sorted(self.len_args.items())), id(self.profile) if self.profile is not None else None)

    def __eq__(self, other):
        return isinstance(other, BinSpec) and self.key() == other.key()

    def __hash__(self):
        return hash(self.key())

    def __repr__(self):
        return f"BinSpec({self.type!r}, {self.len_args!r})"


def as_bin(b):
    """A thin-shell radius (float, physical) or a BinSpec."""
    return b if isinstance(b, BinSpec) else BinSpec("shell", {"R": float(b)})


def multipole_fields_bins(half_spec, J, l, m, bins, box_size, phi_power, out=None, ws=None, bin_major=False):
    """a_lm^b for radial bins of any supported profile (shell, sphere,
    thick_shell, gaussian, gaussian_shell, custom_real, custom_kspace), in the
    layout of multipole_fields (bin_major as there).  The GPU path per bin
    follows radial_multipole_windows.py:269-313: j_l for shells, the analytic
    monopole transfer for l = 0, else a host table of U_l(k)."""
    from . import radial_profiles as rp

    bins = [as_bin(b) for b in bins]
    nb = len(bins)
    L = 1 << J
    g2p = L / float(box_size)
    per_bin = [rp.profile_mode(b.type, b.len_args, l) for b in bins]
    if len(set(per_bin)) > 1:
        # bins on different profile paths: one call per path, its bins
        # gathered into the shared layout
        if out is None:
            out = torch.zeros((nb, L ** 3) if bin_major else (L ** 3, BIN_STRIDE), dtype=torch.complex64,
                              device=half_spec.device)
        for path in dict.fromkeys(per_bin):
            idx = [i for i, p in enumerate(per_bin) if p == path]
            part = multipole_fields_bins(half_spec, J, l, m, [bins[i] for i in idx], box_size, phi_power, ws=ws,
                                         bin_major=bin_major)
            if bin_major:
                out[idx] = part.view(1, L ** 3) if part.dim() == 1 else part
            else:
                out[:, idx] = part.view(L ** 3, 1) if part.dim() == 1 else part[:, :len(idx)]
        return out
    mode = per_bin[0]
    if mode == "shell":
        radii = [(b.len_args["R_shell"] if b.type == "gaussian_shell" else b.len_args["R"]) * g2p for b in bins]
        return multipole_fields(half_spec, J, l, m, radii, phi_power, out=out, ws=ws, bin_major=bin_major)
    dev = half_spec.device
    if out is None:
        out = _fields_out(J, nb, bin_major, dev)
    if ws is None:
        ws = _workspace(fields_ws_bytes(J, nb, bin_major), dev)
    lib = _lib.load()
    if mode == "analytic":
        from .window import WIN_ARGS, WIN_CODES, HermesWindow

        arr = (HermesWindow * nb)()
        for k, b in enumerate(bins):
            arr[k].type = WIN_CODES[b.type]
            for i, nm in enumerate(WIN_ARGS[b.type]):
                arr[k].len[i] = float(b.len_args[nm]) * g2p
            arr[k].los[2] = 1.0
            arr[k].scale = 1.0
        fn = lib.hermes_multipole_fields_window_bm if bin_major else lib.hermes_multipole_fields_window
        _lib.check(fn(_ptr(half_spec), J, int(l), int(m), arr, nb, _ptr(phi_power), _ptr(out), _ptr(ws), ws.numel(),
                      _stream_ptr(dev)), "hermes_multipole_fields_window")
        return out
    k_max = math.sqrt(3.0) * g2p
    tabs = [rp.build_radial_multipole_table(b.type, b.len_args, l, k_max, b.profile) for b in bins]
    sizes = np.array([t.size for _, t in tabs], dtype=np.int32)
    offs = np.concatenate([[0], np.cumsum(sizes[:-1])]).astype(np.int64)
    kms = np.array([km for km, _ in tabs], dtype=np.float64)
    dt = torch.as_tensor(np.concatenate([t for _, t in tabs]), dtype=torch.float64, device=dev)
    fn = lib.hermes_multipole_fields_table_bm if bin_major else lib.hermes_multipole_fields_table
    _lib.check(fn(_ptr(half_spec), J, int(l), int(m), _ptr(dt), offs.ctypes.data_as(ctypes.c_void_p),
                  sizes.ctypes.data_as(ctypes.c_void_p), kms.ctypes.data_as(ctypes.c_void_p), g2p, nb,
                  _ptr(phi_power), _ptr(out), _ptr(ws), ws.numel(), _stream_ptr(dev)),
               "hermes_multipole_fields_table")
    return out  # dt is released in stream order after the table kernel


def complex_full_window_bin(window):
    """(l, m, bin) of a complex full-FFT WindowFunc (io/window.py:198-264):
    legendre_multipole is the thin shell j_l(2 pi k R) Y_lm
    (utils/legendre_windows.py:41-119), radial_multipole any radial profile
    (utils/radial_multipole_windows.py:267-316); both bandwidth 1."""
    if window.bandwidth != 1:
        raise ValueError(f"{window.type} currently supports only bandwidth=1.")
    oa = window.other_args or {}
    try:
        l, m = int(oa["l"]), int(oa["m"])
        if window.type == "radial_multipole":
            return l, m, BinSpec(str(oa["radial_type"]), window.len_args, oa.get("profile_config") or None)
    except KeyError as exc:
        raise ValueError(f"{window.type} missing required other_args key: {exc}") from None
    if window.type != "legendre_multipole":
        raise ValueError(f"Unsupported complex full-FFT window type: {window.type}")
    if window.len_args.get("R") is None:
        raise ValueError("legendre_multipole requires len_args={'R': ...}.")
    return l, m, BinSpec("shell", {"R": float(window.len_args["R"])})


def convolve_complex_full(field, window):
    """SFCField @ a complex full-FFT window: ifftn(fftn(eps) K_lm) as a
    complex64 [L, L, L] device tensor (utils/convolution.py:291-295), from
    the multipole field kernels."""
    l, m, b = complex_full_window_bin(window)
    spec = rfft_field(field.epsilon_device.to(torch.float32).contiguous())
    a = multipole_fields_bins(spec, window.J, l, m, [b], window.box_size, window.phi_power())
    return a.view(window.L, window.L, window.L)


def complex_full_kernel(window):
    """K_lm of a complex full-FFT window as complex64 [L, L, L]: the field
    kernels applied to the half spectrum of a unit impulse (all ones) give
    ifftn(K), and one forward FFT returns K."""
    l, m, b = complex_full_window_bin(window)
    L = window.L
    ones = torch.ones((L, L, L // 2 + 1), dtype=torch.complex64, device=window.device)
    a = multipole_fields_bins(ones, window.J, l, m, [b], window.box_size, window.phi_power())
    return torch.fft.fftn(a.view(L, L, L).to(torch.complex128)).to(torch.complex64)


def multipole_contract(eps1, fields2, nb2, gamma, J, fields3=None, nb3=None, conj_sign=1):
    """S[b2, b3] complex128 (see include/hermes_gb300.h)."""
    nb3 = nb2 if fields3 is None else nb3
    dev = eps1.device
    ws = _workspace(_ws_bytes(J, max(nb2, nb3)), dev)
    out = np.zeros((nb2, nb3, 2), dtype=np.float64)
    g = (ctypes.c_double * 9)(*np.asarray(gamma, dtype=np.float64).ravel())
    _lib.check(_lib.load().hermes_multipole_contract(_ptr(eps1), _ptr(fields2), nb2, _ptr(fields3), nb3,
                                                     int(conj_sign), g, J, out.ctypes.data_as(ctypes.c_void_p),
                                                     _ptr(ws), ws.numel(), _stream_ptr(dev)),
               "hermes_multipole_contract")
    return out[..., 0] + 1j * out[..., 1]


ENGINES = ("tensor", "simt")


def multipole_contract_async(eps1, fields2, nb2, gamma_c, J, dev_out, fields3=None, nb3=None, conj_sign=1,
                             chunk_x=0, ctas_per_sm=0, ws=None, engine="tensor", bin_major=False):
    """hermes_multipole_contract_async: S (times 4 pi / L^3) into the device
    float64 tensor dev_out [16, 16, 2] on the current stream, no host sync.
    gamma_c: a ctypes double[9] (kept alive by the caller during capture).
    engine: 'tensor' (bin x bin product on tcgen05, BF16x3 operands) or 'simt'
    (the all-FP32 CUDA-core kernel).  bin_major: fields in the [nb, L^3]
    layout of multipole_fields(bin_major=True) (tensor engine,
    hermes_multipole_contract_bm_async)."""
    if engine not in ENGINES:
        raise ValueError(f"engine must be one of {ENGINES}")
    if bin_major and engine != "tensor":
        raise ValueError("bin-major fields are read by the tensor engine only")
    nb3 = nb2 if fields3 is None else nb3
    dev = eps1.device
    if ws is None:
        ws = _workspace(_ws_bytes(J, 1 if bin_major else max(nb2, nb3)), dev)
    lib = _lib.load()
    if bin_major:
        fn = lib.hermes_multipole_contract_bm_async
    else:
        fn = lib.hermes_multipole_contract_async if engine == "tensor" else lib.hermes_multipole_contract_simt_async
    _lib.check(fn(_ptr(eps1), _ptr(fields2), nb2, _ptr(fields3), nb3, int(conj_sign), gamma_c, J, int(chunk_x),
                  int(ctas_per_sm), _ptr(dev_out), _ptr(ws), ws.numel(), _stream_ptr(dev)),
               "hermes_multipole_contract_async")
    return dev_out


def contract_status(J, ws=None, device="cuda"):
    """0, or 1 when a bounded wait of the last tensor-core contraction on the
    workspace gave up (its results are then NaN)."""
    if ws is None:
        ws = _workspace(_ws_bytes(J, 1), torch.device(device))
    st = ctypes.c_int(0)
    _lib.check(_lib.load().hermes_multipole_contract_status(_ptr(ws), ws.numel(), J, ctypes.byref(st),
                                                            _stream_ptr(ws.device)), "hermes_multipole_contract_status")
    return st.value


def multipole_contract_engine(eps1, fields2, nb2, gamma, J, fields3=None, nb3=None, conj_sign=1, engine="tensor",
                              chunk_x=0, ctas_per_sm=0, bin_major=False):
    """S[b2, b3] complex128 from a chosen engine (async launch + one read)."""
    nb3 = nb2 if fields3 is None else nb3
    g = (ctypes.c_double * 9)(*np.asarray(gamma, dtype=np.float64).ravel())
    out = torch.zeros((MAX_BINS, MAX_BINS, 2), dtype=torch.float64, device=eps1.device)
    multipole_contract_async(eps1, fields2, nb2, g, J, out, fields3=fields3, nb3=nb3, conj_sign=conj_sign,
                             chunk_x=chunk_x, ctas_per_sm=ctas_per_sm, engine=engine, bin_major=bin_major)
    o = out[:nb2, :nb3].cpu().numpy()
    return o[..., 0] + 1j * o[..., 1]


def multipole_contract_plain(eps1, a2, a3, gamma, J):
    dev = eps1.device
    ws = _workspace(_ws_bytes(J, 1), dev)
    out = np.zeros(2, dtype=np.float64)
    g = (ctypes.c_double * 9)(*np.asarray(gamma, dtype=np.float64).ravel())
    _lib.check(_lib.load().hermes_multipole_contract_plain(_ptr(eps1), _ptr(a2), _ptr(a3), g, J,
                                                           out.ctypes.data_as(ctypes.c_void_p), _ptr(ws),
                                                           ws.numel(), _stream_ptr(dev)),
               "hermes_multipole_contract_plain")
    return complex(out[0], out[1])


class GraphedMultipole:
    """The (l, m) loop of MultipoleEngine.ddd for one (J, radii, l_max) with
    vertices 2 and 3 sharing the field and radii, as ONE CUDA graph: the rFFT
    of the field and, for every (l, m >= 0), hermes_multipole_fields +
    hermes_multipole_contract_async into a device array of S matrices.  The
    graph works on fixed buffers, including its own workspace: run(delta)
    copies the field into them and replays.  The first run does one uncaptured pass (cuFFT plans, workspace,
    kernel attributes) and then captures.  chunk_x / ctas_per_sm are the
    contraction tile choices (see autotune.tune_contract)."""

    def __init__(self, J, box_size, radii_phys, l_max, phi_array, device, phi_resolution=1024, chunk_x=0,
                 ctas_per_sm=0, use_graph=True, pair_degrees=True):
        self.J, self.L, self.box = int(J), 1 << int(J), float(box_size)
        self.dev = torch.device(device)
        self.radii = [float(r) for r in radii_phys]
        if not 1 < len(self.radii) <= MAX_BINS:
            raise ValueError(f"GraphedMultipole needs 2..{MAX_BINS} radii.")
        self.grid = [r * self.L / self.box for r in self.radii]
        self.l_max = int(l_max)
        self.lm = [(l, m) for l in range(self.l_max + 1) for m in range(l + 1)]
        # m = 0 terms of degrees (l, l + 1) from one paired fields pass and contraction
        self.pairs = degree_pairs(self.lm) if pair_degrees else []
        phi = np.asarray(phi_array, dtype=np.float64)
        self.gamma = (ctypes.c_double * 9)(*cal_gamma(phi, phi.shape[0] // phi_resolution, phi_resolution).ravel())
        self.P = phi_power_device(phi, self.L, 1, phi_resolution, self.dev)
        L = self.L
        self.eps = torch.empty((L, L, L), dtype=torch.float32, device=self.dev)
        self.spec = torch.empty((L, L, L // 2 + 1), dtype=torch.complex64, device=self.dev)
        # bin-major fields [nb, L^3], as the inverse FFT leaves them
        self.fields = torch.empty((len(self.grid), L ** 3), dtype=torch.complex64, device=self.dev)
        self.out = torch.zeros((len(self.lm) + len(self.pairs), MAX_BINS, MAX_BINS, 2), dtype=torch.float64,
                               device=self.dev)
        # own workspace: a captured graph must never see the shared one reallocated
        self.ws = torch.empty(max(fields_ws_bytes(self.J, len(self.grid), True), 256), dtype=torch.uint8,
                              device=self.dev)
        self.chunk_x, self.ctas = int(chunk_x), int(ctas_per_sm)
        self.use_graph = bool(use_graph)
        self.graph = None

    def _body(self):
        lib = _lib.load()
        _lib.check(lib.hermes_fft_r2c(_ptr(self.eps), _ptr(self.spec), self.J, _stream_ptr(self.dev)), "hermes_fft_r2c")
        nb = len(self.grid)
        for j, l in enumerate(self.pairs):
            multipole_fields_pair(self.spec, self.J, l, self.grid, self.P, out=self.fields, ws=self.ws)
            multipole_contract_pair_async(self.eps, self.fields, nb, self.gamma, self.J, self.out[len(self.lm) + j],
                                          chunk_x=self.chunk_x, ctas_per_sm=self.ctas, ws=self.ws)
        paired = {(l + d, 0) for l in self.pairs for d in (0, 1)}
        for k, (l, m) in enumerate(self.lm):
            if (l, m) in paired:
                continue
            multipole_fields(self.spec, self.J, l, m, self.grid, self.P, out=self.fields, ws=self.ws, bin_major=True)
            multipole_contract_async(self.eps, self.fields, nb, self.gamma, self.J, self.out[k],
                                     conj_sign=(-1) ** ((l + m) % 2), chunk_x=self.chunk_x,
                                     ctas_per_sm=self.ctas, ws=self.ws, bin_major=True)

    def summands(self, delta):
        """S_lm[i, j] (complex128 [n_lm, nb, nb]) for the field delta."""
        self.eps.copy_(delta.to(torch.float32))
        if not self.use_graph:
            self._body()
        else:
            if self.graph is None:
                self._body()  # uncaptured pass: plans, workspace and attributes exist before capture
                torch.cuda.synchronize(self.dev)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    self._body()
                self.graph = g
            self.graph.replay()
        nb = len(self.grid)
        o = self.out[:, :nb, :nb].cpu().numpy()
        n = len(self.lm)
        S = o[:n, ..., 0] + 1j * o[:n, ..., 1]
        k_of = {lm: k for k, lm in enumerate(self.lm)}
        for j, l in enumerate(self.pairs):
            S[k_of[(l, 0)]] = o[n + j, ..., 0]
            S[k_of[(l + 1, 0)]] = o[n + j, ..., 1]
        return S

    def ddd(self, delta, pairs, l_min=0):
        """DDD_l [n_samples, n_l] for (r12, r13) samples drawn from the radii
        (the same combination as MultipoleEngine.ddd)."""
        S = self.summands(delta)
        idx = {r: i for i, r in enumerate(self.radii)}
        k_of = {lm: k for k, lm in enumerate(self.lm)}
        res = np.zeros((len(pairs), self.l_max - l_min + 1))
        for li, l in enumerate(range(l_min, self.l_max + 1)):
            for s, (a, b) in enumerate(pairs):
                res[s, li] = combine_multipole_m_terms([S[k_of[(l, m)]][idx[a], idx[b]] for m in range(l + 1)], l)
        return res


def combine_multipole_m_terms(m_values, l):
    """corr3pcf_multipoles.py:173-180."""
    coeff = complex(m_values[0])
    for m in range(1, l + 1):
        coeff += ((-1) ** m) * complex(m_values[m])
        coeff += ((-1) ** (-m)) * np.conj(complex(m_values[m]))
    coeff *= (-1) ** l
    return coeff.real


class MultipoleEngine:
    """Batched multipole contraction of three fields over radius pairs."""

    def __init__(self, eps1, eps2, eps3, phi_array, J, box_size, phi_resolution=1024, share23=None,
                 engine="tensor", pair_degrees=True):
        if engine not in ENGINES:
            raise ValueError(f"engine must be one of {ENGINES}")
        self.engine = engine
        # m = 0 terms of degrees (l, l + 1) from one paired fields pass and
        # contraction (summands_shared, tensor engine, thin shells)
        self.pair_degrees = bool(pair_degrees)
        self.bin_major = engine == "tensor"
        self.J = int(J)
        self.L = 1 << self.J
        self.box = float(box_size)
        self.dev = eps1.device
        self.eps1 = eps1.to(torch.float32).contiguous()
        self.spec2 = rfft_field(eps2.to(torch.float32).contiguous())
        same = share23 if share23 is not None else (eps3 is eps2 or (eps3.data_ptr() == eps2.data_ptr()))
        self.same23 = bool(same)
        self.spec3 = self.spec2 if self.same23 else rfft_field(eps3.to(torch.float32).contiguous())
        self.phi = np.asarray(phi_array, dtype=np.float64)
        support = self.phi.shape[0] // phi_resolution
        if support != 3:
            raise NotImplementedError("The GPU contraction is specialised for a support-3 scaling function (db2).")
        self.gamma = cal_gamma(self.phi, support, phi_resolution)
        self.P = phi_power_device(self.phi, self.L, 1, phi_resolution, self.dev)
        self.timing = {"fields_s": 0.0, "contract_s": 0.0}

    def _fields(self, spec, l, m, bins):
        # the tensor engine reads the bin-major layout the inverse FFT writes
        return multipole_fields_bins(spec, self.J, l, m, bins, self.box, self.P, bin_major=self.bin_major)

    def summands_shared(self, lms, bins):
        """S_lm[i, j] for every (l, m) in lms over one list of at most 16 bins
        shared by vertices 2 and 3 (a_{l,-m} from the conjugate of a_lm),
        complex128 [len(lms), nb, nb]: every fields pass and contraction is
        queued on the current stream into one device array, which is read
        back once (no host round trip per (l, m)).  With the tensor engine
        and thin-shell bins, the m = 0 terms of degrees (l, l + 1), l even,
        share one paired fields pass and contraction (degree_pairs)."""
        bins = [as_bin(b) for b in bins]
        nb = len(bins)
        if not (self.same23 and 1 <= nb <= MAX_BINS):
            raise ValueError("summands_shared needs vertices 2 and 3 to share the field and 1..16 bins")
        g = (ctypes.c_double * 9)(*np.asarray(self.gamma, dtype=np.float64).ravel())
        k_of = {lm: k for k, lm in enumerate(lms)}
        pairs = self._degree_pairs(lms, bins)
        paired = {(l + d, 0) for l in pairs for d in (0, 1)}
        out = torch.zeros((len(lms) + len(pairs), MAX_BINS, MAX_BINS, 2), dtype=torch.float64, device=self.dev)
        t0 = time.perf_counter()
        for j, l in enumerate(pairs):
            f = multipole_fields_pair(self.spec2, self.J, l, self._grid(bins), self.P)
            multipole_contract_pair_async(self.eps1, f, nb, g, self.J, out[len(lms) + j])
            del f
        for k, (l, m) in enumerate(lms):
            if (l, m) in paired:
                continue
            f = self._fields(self.spec2, l, m, bins)
            multipole_contract_async(self.eps1, f, nb, g, self.J, out[k], conj_sign=(-1) ** ((l + m) % 2),
                                     engine=self.engine, bin_major=self.bin_major)
            del f  # released in stream order, after the contraction that reads it
        o = out[:, :nb, :nb].cpu().numpy()
        # the fields passes and contractions run queued together; their time
        # is counted under contract_s
        self.timing["contract_s"] += time.perf_counter() - t0
        S = o[:len(lms), ..., 0] + 1j * o[:len(lms), ..., 1]
        for j, l in enumerate(pairs):
            S[k_of[(l, 0)]] = o[len(lms) + j, ..., 0]
            S[k_of[(l + 1, 0)]] = o[len(lms) + j, ..., 1]
        return S

    def _grid(self, bins):
        """Thin-shell radii of bins in grid units."""
        g2p = self.L / self.box
        return [(b.len_args["R_shell"] if b.type == "gaussian_shell" else b.len_args["R"]) * g2p for b in bins]

    def _degree_pairs(self, lms, bins):
        """degree_pairs(lms) where the paired kernels apply: tensor engine,
        thin-shell bins."""
        if not (self.bin_major and self.pair_degrees):
            return []
        from . import radial_profiles as rp

        return [l for l in degree_pairs(lms)
                if all(rp.profile_mode(b.type, b.len_args, d) == "shell" for b in bins for d in (l, l + 1))]

    def summands(self, l, m, r12_phys, r13_phys):
        """S_m[i, j] for two lists of radial bins (thin-shell radii in physical
        units, or BinSpec), complex128 [n12, n13]."""
        b12 = [as_bin(r) for r in r12_phys]
        b13 = [as_bin(r) for r in r13_phys]
        out = np.zeros((len(b12), len(b13)), dtype=np.complex128)
        shared = self.same23 and b12 == b13
        for i0 in range(0, len(b12), MAX_BINS):
            c12 = b12[i0:i0 + MAX_BINS]
            t0 = time.perf_counter()
            f2 = self._fields(self.spec2, l, m, c12)
            for j0 in range(0, len(b13), MAX_BINS):
                c13 = b13[j0:j0 + MAX_BINS]
                if shared and i0 == j0:
                    t1 = time.perf_counter()
                    self.timing["fields_s"] += t1 - t0
                    S = multipole_contract_engine(self.eps1, f2, len(c12), self.gamma, self.J,
                                                  conj_sign=(-1) ** ((l + m) % 2), engine=self.engine,
                                                  bin_major=self.bin_major)
                else:
                    f3 = self._fields(self.spec3, l, -m, c13)
                    t1 = time.perf_counter()
                    self.timing["fields_s"] += t1 - t0
                    S = multipole_contract_engine(self.eps1, f2, len(c12), self.gamma, self.J, fields3=f3,
                                                  nb3=len(c13), engine=self.engine, bin_major=self.bin_major)
                    del f3
                self.timing["contract_s"] += time.perf_counter() - t1
                t0 = time.perf_counter()
                out[i0:i0 + len(c12), j0:j0 + len(c13)] = S
            del f2
        return out

    def ddd(self, pairs, l_min, l_max):
        """DDD_l for samples given as (r12, r13) physical radii -> [n_samples, n_l]."""
        pairs = [(as_bin(a), as_bin(b)) for a, b in pairs]

        def order(bins):
            return sorted(set(bins), key=lambda b: (b.type, sorted(b.len_args.items()), str(b.key()[2])))

        r12 = order(p[0] for p in pairs)
        r13 = order(p[1] for p in pairs)
        i12 = {r: i for i, r in enumerate(r12)}
        i13 = {r: i for i, r in enumerate(r13)}
        if self.same23 and r12 != r13:
            both = order(list(r12) + list(r13))
            r12 = r13 = both
            i12 = i13 = {r: i for i, r in enumerate(both)}
        res = np.zeros((len(pairs), l_max - l_min + 1))
        shared = None
        if self.same23 and r12 == r13 and len(r12) <= MAX_BINS:
            lms = [(l, m) for l in range(l_min, l_max + 1) for m in range(l + 1)]
            S = self.summands_shared(lms, r12)
            shared = {lm: S[k] for k, lm in enumerate(lms)}
        for li, l in enumerate(range(l_min, l_max + 1)):
            if shared is not None:
                Sm = [shared[(l, m)] for m in range(0, l + 1)]
            else:
                Sm = [self.summands(l, m, r12, r13) for m in range(0, l + 1)]
            for s, (a, b) in enumerate(pairs):
                res[s, li] = combine_multipole_m_terms([Sm[m][i12[a], i13[b]] for m in range(l + 1)], l)
        return res

    def ddd_plain(self, pairs, l_min, l_max):
        """The per-sample reference form: both side fields rebuilt per sample
        and (l, m), reference-order contraction of one pair."""
        res = np.zeros((len(pairs), l_max - l_min + 1))
        for s, (a, b) in enumerate(pairs):
            a, b = as_bin(a), as_bin(b)
            for li, l in enumerate(range(l_min, l_max + 1)):
                vals = []
                for m in range(0, l + 1):
                    f2 = self._fields(self.spec2, l, m, [a])
                    f3 = self._fields(self.spec3, l, -m, [b])
                    vals.append(multipole_contract_plain(self.eps1, f2, f3, self.gamma, self.J))
                    del f2, f3
                res[s, li] = combine_multipole_m_terms(vals, l)
        return res


def legendre_triple_coeff(l, lp, k):
    """utils/special_functions.py:337-363."""
    from math import lgamma

    s = l + lp + k
    if (k > l + lp) or (k < abs(l - lp)) or (s % 2 != 0):
        return 0.0
    g = s // 2
    log_val = (lgamma(s - 2 * l + 1) + lgamma(s - 2 * lp + 1) + lgamma(s - 2 * k + 1) - lgamma(s + 2)
               + 2 * (lgamma(g + 1) - lgamma(g - l + 1) - lgamma(g - lp + 1) - lgamma(g - k + 1)))
    return float((2 * k + 1) * np.exp(log_val))


_GAUNT = {}


def _gaunt_device(n, device):
    key = (n, str(device))
    g = _GAUNT.get(key)
    if g is None:
        G = np.zeros((n, n, n))
        for k in range(n):
            for l in range(n):
                for lp in range(n):
                    G[k, l, lp] = legendre_triple_coeff(l, lp, k)
        g = torch.as_tensor(G, device=device)
        _GAUNT[key] = g
    return g


def mixing_solve(A, B, lmax, device="cuda"):
    """zeta_l for A(mu) = B(mu) C(mu) (special_functions.py:366-409), float64
    on the GPU for all samples at once (hermes_mixing_solve).  A, B:
    [n_samples, >= lmax+1].  Returns (C, M, cond) as numpy arrays."""
    A = np.atleast_2d(np.asarray(A, dtype=np.float64))
    B = np.atleast_2d(np.asarray(B, dtype=np.float64))
    n = lmax + 1
    if A.shape[1] < n or B.shape[1] < n:
        raise ValueError("A and B must have length at least lmax+1.")
    A, B = A[:, :n], B[:, :n]
    if np.any(B[:, 0] == 0):
        raise ValueError("B[0] is zero.")
    ns = A.shape[0]
    At = torch.as_tensor(np.ascontiguousarray(A), device=device)
    Bt = torch.as_tensor(np.ascontiguousarray(B), device=device)
    C = torch.empty((ns, n), dtype=torch.float64, device=device)
    M = torch.empty((ns, n, n), dtype=torch.float64, device=device)
    cond = torch.empty(ns, dtype=torch.float64, device=device)
    _lib.check(_lib.load().hermes_mixing_solve(_ptr(At), _ptr(Bt), _ptr(_gaunt_device(n, At.device)), ns, n,
                                               _ptr(C), _ptr(M), _ptr(cond), _stream_ptr(At.device)),
               "hermes_mixing_solve")
    return C.cpu().numpy(), M.cpu().numpy(), cond.cpu().numpy()


class Corr3PCFMultipoleData(ResultFileIO):
    """Result container (pyhermes/io/corr3pcf_multipole.py:9-30).  The file
    written by ``save_corr3pcf_multipole`` / read by
    ``load_corr3pcf_multipole`` is the reference's NumPy-framed pickle with
    the same top-level keys and order (``timing`` stays in memory)."""

    FILE_KEYS = ("sfc_info1", "sfc_info2", "sfc_info3", "corr3pcf_multipole_info", "sample_params",
                 "binning_window12", "binning_window13", "r12", "r13", "l", "ddd_l", "rrr_l", "delta_ddd_l",
                 "zeta_l", "zeta_condition")

    _OWN_SAVE, _OWN_LOAD = "save_corr3pcf_multipole", "load_corr3pcf_multipole"

    def __init__(self, data_path=None):
        for k in self.FILE_KEYS:
            setattr(self, k, None)
        self.corr3pcf_multipole_info = {}
        self.timing = {}
        if data_path:
            self.load_corr3pcf_multipole(data_path)

    def save_corr3pcf_multipole(self, f_out, overwrite=False):
        f_out = check_fout(self, f_out, overwrite)
        if not f_out:
            return None
        with open(f_out, "wb") as f:
            write_numpy_pickle(f, {k: getattr(self, k) for k in self.FILE_KEYS})
        return f_out

    def load_corr3pcf_multipole(self, f_in):
        with open(f_in, "rb") as f:
            d = read_numpy_pickle(f)
        for k in self.FILE_KEYS:
            setattr(self, k, d.get(k))
        self.corr3pcf_multipole_info = d.get("corr3pcf_multipole_info") or {}


PRODUCTS = ("ddd_l", "rrr_l", "delta_ddd_l", "zeta_l")


class Corr_3PCF_Multipole:
    task_name = "Corr_3PCF_Multipole"

    def __init__(self, param_task=None, device="cuda"):
        self.task_params = task_params(self.task_name, param_task)
        self.device = torch.device(device)
        self.format_params()

    def format_params(self):
        """The task parameters into attributes (theory/corr3pcf_multipole.py:60-160); call again after
        editing task_params."""
        tp = self.task_params
        self.sfc_field = tp.get("sfc_field", "")
        for i in (1, 2, 3):
            setattr(self, f"sfc_field{i}", tp.get(f"sfc_field{i}", "") or self.sfc_field)
        self.random = tp.get("random")
        for i in (1, 2, 3):
            r = tp.get(f"random{i}")
            setattr(self, f"random{i}", self.random if r in (None, "") else r)
        self.weight_normalization = normalize_task_weight_normalization(tp.get("weight_normalization", "catalog"))
        window = tp.get("window")
        self.window = window if (isinstance(window, dict) and window.get("type")) else None
        for i in (1, 2, 3):
            wi = tp.get(f"window{i}")
            wi = wi if (isinstance(wi, dict) and wi.get("type")) else None
            setattr(self, f"window{i}", wi or (dict(self.window) if self.window else None))
        self.sampling = self._normalize_sampling(tp.get("sampling"))
        self.samples = self._expand_sampling(self.sampling)
        t12 = self.binning_window12_template = self._edge_template(tp.get("binning_window12"), "binning_window12")
        t13 = self.binning_window13_template = self._edge_template(tp.get("binning_window13"), "binning_window13")
        self.binning_window12 = [self._sample_window(t12, s, "binning_window12") for s in self.samples]
        self.binning_window13 = [self._sample_window(t13, s, "binning_window13") for s in self.samples]
        self.l_min = int(tp["l_min"])
        self.l_max = int(tp["l_max"])
        if self.l_min < 0 or self.l_max < 0 or self.l_min > self.l_max:
            raise ValueError("Corr_3PCF_Multipole requires 0 <= l_min <= l_max.")
        backend = str(tp.get("summation_backend", "gb300")).strip().lower()
        self._backend_given = backend
        if backend not in {"gb300", "gpu", "plain", "cpu"}:
            raise ValueError("summation_backend must be 'gb300', 'gpu', 'plain' or 'cpu'.")
        self.summation_backend = "plain" if backend == "plain" else "gb300"
        self.contraction_engine = str(tp.get("contraction_engine", "tensor")).strip().lower()
        if self.contraction_engine not in ENGINES:
            raise ValueError(f"contraction_engine must be one of {ENGINES}.")
        prods = tp.get("products", "zeta_l")
        prods = [prods] if isinstance(prods, str) else list(prods)
        self.products = []
        for p in prods:
            p = str(p).strip().lower()
            if p not in PRODUCTS:
                raise ValueError(f"Unsupported product '{p}'.")
            if p not in self.products:
                self.products.append(p)
        self.fout_path = tp.get("fout_path", "")
        self.zeta_condition_warning = float(tp.get("zeta_condition_warning", 1.0e12))
        if not np.isfinite(self.zeta_condition_warning) or self.zeta_condition_warning <= 0.0:
            raise ValueError("zeta_condition_warning must be a finite positive number.")
        self._fields_prepared = False

    def _resolution_diagnostics(self):
        """theory/corr3pcf_multipole.py:621-665: per binning edge, the smallest
        radial scale against l_max (pi R / dx; a warning when
        l_max / (pi R / dx) >= 0.7)."""
        out = []
        if self.l_max == 0:
            return out
        keys = {"shell": "R", "thick_shell": "R", "sphere": "R", "gaussian": "R", "gaussian_shell": "R_shell"}
        ref = self.reference
        for name, windows in (("binning_window12", self.binning_window12), ("binning_window13", self.binning_window13)):
            kind = str(windows[0]["type"]).strip().lower()
            if kind not in keys:
                continue
            radii = np.asarray([float(w["len_args"][keys[kind]]) for w in windows], dtype=np.float64)
            pos = radii[radii > 0.0]
            if pos.size == 0:
                continue
            q = float(np.pi * pos.min() * ref.L / ref.box_size)
            ratio = float(self.l_max / q)
            out.append({"edge": name, "radial_type": kind, "min_radius": float(pos.min()),
                        "max_radius": float(pos.max()), "q_grid_min": q, "l_max_over_q_grid_min": ratio})
            if ratio >= 0.7:
                logger.warning("Multipole resolution diagnostic | %s: l_max=%d, min radial scale=%.6g, pi R / dx=%.3f, "
                               "l_max/(pi R/dx)=%.3f. The highest multipoles are close to the grid high-k range; "
                               "check J convergence.", name, self.l_max, pos.min(), q, ratio)
        return out

    def _radial_profile_diagnostics(self):
        """theory/corr3pcf_multipole.py:668-718: every tabulated radial
        window of both edges checked per sample and l (from l_min, or 1 for
        built-in profiles whose monopole is analytic), with a warning for a
        table that misses the tolerance."""
        from .radial_profiles import diagnose_radial_multipole_table

        out = []
        tp = self.task_params
        if not bool(tp.get("radial_profile_diagnostics", True)):
            return out
        tol = float(tp.get("radial_profile_diagnostic_tolerance", 1e-5))
        probes = int(tp.get("radial_profile_diagnostic_probes", 33))
        k_max = float(np.sqrt(3.0) * self.reference.L / self.reference.box_size)
        for name, windows in (("binning_window12", self.binning_window12), ("binning_window13", self.binning_window13)):
            for idx, params in enumerate(windows):
                kind = str(params["type"]).strip().lower()
                if kind == "shell" or (kind == "gaussian_shell" and float(params["len_args"]["R_smooth"]) == 0.0):
                    continue
                first = self.l_min if kind.startswith("custom_") else max(1, self.l_min)
                for l in range(first, self.l_max + 1):
                    d = diagnose_radial_multipole_table(kind, params["len_args"], l, k_max,
                                                        profile_config=params.get("other_args", {}), tolerance=tol,
                                                        probe_count=probes)
                    d.update({"edge": name, "sample_idx": int(idx)})
                    out.append(d)
                    if not d["passed"]:
                        logger.warning("Radial profile diagnostic exceeded tolerance | %s[%d], type=%s, l=%d, "
                                       "tolerance=%.3e. Increase profile quadrature/table points or verify the "
                                       "profile support.", name, idx, kind, l, tol)
        return out

    def _info_snapshot(self, expanded):
        """corr3pcf_multipole_info with the reference's keys
        (theory/corr3pcf_multipole.py:767 and the task parameters)."""
        tp = self.task_params
        info = {"sfc_field": describe_input(self.sfc_field)}
        for i in (1, 2, 3):
            info[f"sfc_field{i}"] = describe_input(getattr(self, f"sfc_field{i}"))
        info["random"] = describe_input(tp.get("random"))
        for i in (1, 2, 3):
            info[f"random{i}"] = describe_input(self.rand.get(i, getattr(self, f"random{i}", None)))
        info.update({"weight_normalization": self.weight_normalization, "window": describe_input(self.window)})
        for i in (1, 2, 3):
            info[f"window{i}"] = describe_input(getattr(self, f"window{i}"))
        sampling = {"mode": self.sampling["mode"],
                    "values": {k: [float(x) for x in v] for k, v in self.sampling["values"].items()}}
        info.update({"binning_window12_template": describe_input(self.binning_window12_template),
                     "binning_window13_template": describe_input(self.binning_window13_template),
                     "sampling": sampling, "n_samples": len(self.samples), "l_min": self.l_min, "l_max": self.l_max,
                     "gpu_device_id": int(tp.get("gpu_device_id", 0) or 0),
                     "gpu_threads_per_block": list(tp.get("gpu_threads_per_block") or [8, 8, 8]),
                     "summation_backend": self._backend_given, "execution_mode": "serial",
                     "sample_mpi": {"ranks_per_sample": 1, "gpu_device_ids": []},
                     "cache_multipole_fields": False, "cache_dir": "", "verbose_m_progress": False,
                     "verbose_profile": False, "zeta_condition_warning": self.zeta_condition_warning,
                     "threads": int(tp.get("threads", 1) or 1), "products": list(self.products),
                     "radial_profile_diagnostics": bool(tp.get("radial_profile_diagnostics", True)),
                     "radial_profile_diagnostic_tolerance": float(tp.get("radial_profile_diagnostic_tolerance", 1e-5)),
                     "radial_profile_diagnostic_probes": int(tp.get("radial_profile_diagnostic_probes", 33)),
                     "expanded_products": list(expanded),
                     "resolution_diagnostics": self._resolution_diagnostics(),
                     "radial_profile_diagnostics_result": list(getattr(self, "radial_profile_diagnostics", [])),
                     "rho_vertices": list(getattr(self, "rho_vertices", [None, None, None])),
                     "fout_path": self.fout_path})
        return info

    # ---- sampling (corr3pcf_multipole.py:229-322) ----------------------------
    def _normalize_sampling(self, sampling):
        if not isinstance(sampling, dict):
            raise TypeError("Corr_3PCF_Multipole requires a 'sampling' dictionary.")
        s = copy.deepcopy(sampling)
        mode = str(s.pop("mode", "grid")).strip().lower()
        if mode not in {"grid", "paired"}:
            raise ValueError("sampling.mode must be 'grid' or 'paired'.")
        values = {}
        for name, spec in s.items():
            if isinstance(spec, dict):
                if "values" in spec:
                    v = np.asarray(spec["values"], dtype=np.float64)
                elif {"min", "max", "n"}.issubset(spec):
                    v = np.linspace(float(spec["min"]), float(spec["max"]), int(spec["n"]))
                elif {"start", "stop", "step"}.issubset(spec):
                    st = float(spec["step"])
                    v = np.arange(float(spec["start"]), float(spec["stop"]) + 0.5 * st, st)
                else:
                    raise ValueError(f"sampling.{name} must use 'values', 'min/max/n', 'start/stop/step'.")
            elif isinstance(spec, (list, tuple, np.ndarray)):
                v = np.asarray(spec, dtype=np.float64)
            else:
                v = np.asarray([spec], dtype=np.float64)
            values[name] = v
        if not values:
            raise ValueError("sampling must contain at least one sampled parameter.")
        return {"mode": mode, "values": values}

    def _expand_sampling(self, sampling):
        values = sampling["values"]
        names = list(values)
        if sampling["mode"] == "grid":
            return [{n: float(v) for n, v in zip(names, combo)}
                    for combo in itertools.product(*(values[n] for n in names))]
        n = max(a.size for a in values.values())
        if any(a.size not in (1, n) for a in values.values()):
            raise ValueError("sampling.mode='paired' requires each parameter to have length 1 or the shared length.")
        return [{k: float(a[0] if a.size == 1 else a[i]) for k, a in values.items()} for i in range(n)]

    @staticmethod
    def _edge_template(value, name):
        """theory/corr3pcf_multipole.py:205-227: a binning-window template
        with a non-empty (lower-cased) type and dict len_args / other_args /
        mapping (None read as empty)."""
        if not isinstance(value, dict):
            raise TypeError(f"{name} must be a dictionary.")
        if not value.get("type"):
            raise ValueError(f"{name} must define a non-empty 'type'.")
        params = copy.deepcopy(value)
        params["type"] = str(params["type"]).strip().lower()
        for key in ("len_args", "other_args", "mapping"):
            if params.get(key) is None:
                params[key] = {}
            if not isinstance(params[key], dict):
                raise TypeError(f"{name}.{key} must be a dictionary.")
        return params

    def _sample_window(self, template, sample, name="binning window"):
        """theory/corr3pcf_multipole.py:296-324: mapping targets 'X' or
        'len_args.X' / 'other_args.X' take a sampling parameter (by name)
        or a number."""
        params = copy.deepcopy(template)
        mapping = params.pop("mapping", {}) or {}
        params["len_args"] = copy.deepcopy(params.get("len_args", {}) or {})
        params["other_args"] = copy.deepcopy(params.get("other_args", {}) or {})
        for target, source in mapping.items():
            if isinstance(source, str):
                if source not in sample:
                    raise KeyError(f"Sampling parameter '{source}' is not defined.")
                value = float(sample[source])
            else:
                value = float(source)
            if "." in target:
                sec, key = target.split(".", 1)
                if sec not in ("len_args", "other_args"):
                    raise ValueError(f"Unsupported binning-window mapping target '{target}'.")
                params.setdefault(sec, {})[key] = value
            else:
                params["len_args"][target] = value
        if not params["len_args"]:
            raise ValueError(f"{name} produced an empty len_args dictionary.")
        return params

    # ---- inputs ----------------------------------------------------------------
    def _resolve(self, value, what):
        if isinstance(value, SFCField):
            return value
        if isinstance(value, str) and value:
            return SFCField(data_path=value, device=self.device)
        raise ValueError(f"Missing usable input for {what}.")

    def _normalized(self, field):
        self._density_physical_scale = float(field.scale_factor) ** 3
        if self.weight_normalization == "unit":
            return field.with_normalization("unit")
        if getattr(field, "field_kind", None) != "catalog_field":
            return field.copy()
        return field.switch_weight_normalization(self.weight_normalization)

    def _expanded(self):
        out = list(self.products)
        if "zeta_l" in out:
            for d in ("delta_ddd_l", "rrr_l"):
                if d not in out:
                    out.append(d)
        return out

    def prepare_input_fields(self):
        exp = self._expanded()
        needs_data = any(p in exp for p in ("ddd_l", "delta_ddd_l", "zeta_l"))
        needs_random = any(p in exp for p in ("rrr_l", "delta_ddd_l", "zeta_l"))
        self.data, self.rand = {}, {}
        ref = self._normalized(self._resolve(self.sfc_field1, "field vertex 1"))
        self.reference = ref
        self.rho = ref.field_mean_density(value_unit="grid")
        # per-vertex density of the normalised field before its window
        # (theory/corr3pcf_multipole.py:884-888)
        self.rho_vertices = [self.rho, self.rho, self.rho]
        normalized = {}
        for i in (1, 2, 3):
            if needs_data:
                base = self._normalized(self._resolve(getattr(self, f"sfc_field{i}"), f"field vertex {i}"))
                normalized[i] = base
                self.rho_vertices[i - 1] = base.field_mean_density(value_unit="grid")
                w = getattr(self, f"window{i}")
                self.data[i] = base @ WindowFunc(w, base.sfc_info, device=self.device) if w else base.copy()
            if needs_random:
                r = getattr(self, f"random{i}")
                if r is None or r == "":
                    raise ValueError(f"Missing input for random vertex {i}.")
                if r == "uniform":
                    self.rand[i] = self._uniform_random_after_window(normalized.get(i, ref), self.rho_vertices[i - 1],
                                                                     getattr(self, f"window{i}"), i)
                else:
                    base = self._normalized(self._resolve(r, f"random vertex {i}"))
                    w = getattr(self, f"window{i}")
                    self.rand[i] = base @ WindowFunc(w, base.sfc_info, device=self.device) if w else base.copy()
        self.radial_profile_diagnostics = self._radial_profile_diagnostics()
        self._fields_prepared = True

    def _uniform_random_after_window(self, base, rho, w, vertex):
        """A uniform random vertex after the vertex's window
        (theory/corr3pcf_multipole.py:587-619): the density itself when
        there is no window or W(0) = 1, else a uniform field of that density
        convolved with the window."""
        if not w:
            return float(rho)
        win = WindowFunc(w, base.sfc_info, device=self.device)
        z = complex(np.asarray(win.as_array())[0, 0, 0])
        if abs(z.imag) <= 1e-12 * max(1.0, abs(z.real)) and np.isclose(z.real, 1.0, rtol=1e-10, atol=1e-12):
            return float(rho)
        field = base._spawn_like()
        field.epsilon = torch.full((base.L,) * 3, float(rho), dtype=torch.float32, device=self.device)
        field.sfc_info.update({
            "catalog_weight_sum": None, "catalog_weight_sq_sum": None, "raw_field_weighted_sum": None,
            "field_integral": float(rho) * float(base.V), "weight_normalization": None, "particle_count": None,
            "particle_data_retrievable": False, "particle_data_path": "", "particle_data_format": "",
            "field_kind": "derived_field", "uniform_random_materialized": True, "uniform_random_vertex": int(vertex),
        })
        field.format_sfc_params()
        return field @ win

    def _eps(self, product, i):
        if product == "ddd_l":
            return self.data[i].epsilon_device.to(torch.float32)
        if product == "delta_ddd_l":
            r = self.rand[i]
            d = self.data[i].epsilon_device.double()
            if isinstance(r, float):
                return (d - r).to(torch.float32)
            return (d - r.epsilon_device.double()).to(torch.float32)
        r = self.rand[i]
        if isinstance(r, float):
            return torch.full((self.reference.L,) * 3, r, dtype=torch.float32, device=self.device)
        return r.epsilon_device.to(torch.float32)

    def _pairs(self):
        """(bin12, bin13) per sample: thin-shell radii as floats, other radial
        profiles as BinSpec (type, physical len_args, other_args)."""
        from .radial_profiles import SUPPORTED

        pairs = []
        for w12, w13 in zip(self.binning_window12, self.binning_window13):
            sides = []
            for w in (w12, w13):
                kind = str(w.get("type", "shell")).strip().lower()
                if kind not in SUPPORTED:
                    raise ValueError(f"Unsupported radial profile '{kind}'.")
                la = w.get("len_args", {}) or {}
                sides.append(float(la["R"]) if kind == "shell" else
                             BinSpec(kind, la, (w.get("other_args") or None)))
            pairs.append(tuple(sides))
        return pairs

    def run(self, save_result=True, overwrite=False):
        t0 = time.perf_counter()
        if not self._fields_prepared:
            self.prepare_input_fields()
        exp = self._expanded()
        data = Corr3PCFMultipoleData()
        data.l = np.arange(self.l_min, self.l_max + 1, dtype=np.int32)
        data.binning_window12 = self.binning_window12
        data.binning_window13 = self.binning_window13
        names = list(self.samples[0])
        data.sample_params = {n: np.asarray([s[n] for s in self.samples]) for n in names}
        data.r12 = data.sample_params.get("r12")
        data.r13 = data.sample_params.get("r13")
        pairs = self._pairs()
        scale = float(getattr(self, "_density_physical_scale", 1.0)) ** 3
        ref = self.reference
        phi = ref.sfc_info.get("phi_array")
        if phi is None:
            phi = sample_scaling_function(ref.wavelet_mode, ref.wavelet_level)
        for product in exp:
            if product == "zeta_l":
                continue
            if product == "rrr_l" and all(isinstance(self.rand[i], float) for i in (1, 2, 3)):
                vals = np.zeros((len(pairs), self.l_max - self.l_min + 1))
                if self.l_min == 0:
                    vals[:, 0] = self.rand[1] * self.rand[2] * self.rand[3]
                setattr(data, product, vals * scale)
                continue
            e1, e2, e3 = (self._eps(product, i) for i in (1, 2, 3))
            same23 = (self.sfc_field2 is self.sfc_field3 or self.sfc_field2 == self.sfc_field3) and \
                self.window2 == self.window3 and (product != "delta_ddd_l" or self.random2 == self.random3)
            eng = MultipoleEngine(e1, e2, e2 if same23 else e3, phi, ref.J, ref.box_size, ref.phi_resolution,
                                  share23=same23, engine=self.contraction_engine)
            if self.summation_backend == "plain":
                vals = eng.ddd_plain(pairs, self.l_min, self.l_max)
            else:
                vals = eng.ddd(pairs, self.l_min, self.l_max)
            data.timing[product] = dict(eng.timing)
            setattr(data, product, vals * scale)
        if "zeta_l" in exp:
            if self.l_min != 0:
                raise ValueError("zeta_l requires l_min = 0.")
            z, _, cond = mixing_solve(data.delta_ddd_l, data.rrr_l, self.l_max, device=self.device)
            data.zeta_l = z
            data.zeta_condition = cond
            # theory/corr3pcf_multipole.py:1580-1589
            bad = np.where(cond > self.zeta_condition_warning)[0]
            if bad.size:
                logger.warning("zeta_l mixing matrices exceed zeta_condition_warning=%.3e for samples %s.",
                               self.zeta_condition_warning, bad.tolist())
            logger.info("zeta_l solved from multipole ratio | mixing matrix cond range=[%.3e, %.3e]",
                        float(np.min(cond)), float(np.max(cond)))
        for i in (1, 2, 3):
            if i in self.data:
                setattr(data, f"sfc_info{i}", self.data[i].sfc_info)
        data.corr3pcf_multipole_info = self._info_snapshot(exp)
        self.corr3pcf_multipole_data = data
        if save_result and self.fout_path:
            data.save_corr3pcf_multipole(self.fout_path, overwrite=overwrite)
        logger.info("Corr_3PCF_Multipole %d samples l<=%d in %.3f s", len(pairs), self.l_max, time.perf_counter() - t0)
        return data
