"""The reference's module-level kernel seams, with the reference's signatures.

A maintainer who keeps the reference task classes and swaps only the kernels
re-binds these names as module attributes, e.g.::

    import pyhermes.utils.wavelet_grid as wg
    from pyhermes_gb300 import seams
    wg.project_scaling_grid_numba = seams.project_scaling_grid_numba

Each function keeps the reference's parameter names, argument meaning,
return type and validation errors, accepts the reference's own objects
(fields with a NumPy ``.epsilon``, window objects with ``window_params`` or
``as_array()``, binning windows as parameter dicts) as well as this
package's, and runs on the current CUDA device through the C ABI:

==============================================================  =====================================
reference seam                                                   GPU path
==============================================================  =====================================
utils/wavelet_grid.py:59-70 ``project_scaling_grid_numba``       ``hermes_deposit``
utils/wavelet_grid.py:144-186 ``interpolate_grid_at_pos_numba``  ``hermes_interp``
utils/convolution.py:284-288 ``specialized_convolution_3d``      ``hermes_fft_r2c`` /
                                                                 ``hermes_spectrum_multiply`` /
                                                                 ``hermes_fft_c2r``
theory/corr2pcf.py:366-372 ``pair_product_with_window``          ``hermes_fft_r2c`` +
                                                                 ``hermes_pair_products``
utils/corr3pcf_multipoles.py:460-579 ``calc_DDD_multipole``      the batched multipole engine
utils/special_functions.py:392-409 ``solve_multipoles_from_ratio``  ``hermes_mixing_solve``
theory/corr3pcf.py:68-122 ``estimate_triplet_product_with_sampled_centers``  ``hermes_mc_triplets``
utils/corr3pcf_multipoles.py:393-457 ``compute_multipole_m_summand``  ``hermes_multipole_contract_plain``
==============================================================  =====================================

Fields go to the device as float32 (the arithmetic type of this package);
results come back as float64 NumPy values, as the reference returns them.
``threads``, ``gpu_device_id``, ``gpu_threads_per_block`` and the cache
arguments are accepted for signature compatibility; the work runs on the
current CUDA device and nothing is cached on disk.
"""

import time

import numpy as np
import torch

from . import _lib, kernels
from .kernels import _ptr, _stream_ptr

__all__ = ["project_scaling_grid_numba", "interpolate_grid_at_pos_numba", "specialized_convolution_3d",
           "pair_product_with_window", "calc_DDD_multipole", "solve_multipoles_from_ratio",
           "estimate_triplet_product_with_sampled_centers", "compute_multipole_m_summand"]


def _device():
    return torch.device("cuda", torch.cuda.current_device())


def _level(n):
    n = int(n)
    if n < 2 or n & (n - 1):
        raise ValueError(f"grid size must be a power of two, got {n}")
    return n.bit_length() - 1


def _field_eps(field):
    """float32 device copy of a field: a tensor, an array, or an object with
    ``epsilon_device`` (this package) or ``epsilon`` (the reference)."""
    if isinstance(field, torch.Tensor):
        t = field
    elif isinstance(field, np.ndarray):
        t = torch.as_tensor(field)
    elif getattr(field, "epsilon_device", None) is not None:
        t = field.epsilon_device
    else:
        eps = getattr(field, "epsilon", None)
        if eps is None:
            raise ValueError("field has no epsilon data")
        t = torch.as_tensor(np.asarray(eps))
    if t.is_complex():
        raise TypeError("a real field is required")
    return t.to(device=_device(), dtype=torch.float32).contiguous()


def _field_meta(field):
    """(J, box_size, phi_array, phi_resolution) of a field object."""
    info = getattr(field, "sfc_info", None) or {}

    def get(name, default=None):
        v = getattr(field, name, None)
        return info.get(name, default) if v is None else v

    J = get("J")
    if J is None:
        J = _level(np.asarray(field.epsilon).shape[0])
    phi = get("phi_array")
    if phi is None:
        from .phi import sample_scaling_function

        phi = sample_scaling_function(get("wavelet_mode", "db2"), get("wavelet_level", 10))
    return int(J), float(get("box_size", 1000.0)), np.asarray(phi, dtype=np.float64), int(get("phi_resolution", 1024))


def project_scaling_grid_numba(positions, weights, phi_array, phi_resolution=1024, J=8, box_size=1000.0):
    """eps[x - sx, y - sy, z - sz] += w phi(fx + res sx) phi(fy + res sy)
    phi(fz + res sz) over the 27 stencil points, periodic: float64 [L, L, L].
    The sum is an int64 fixed-point accumulation (the same field for any
    particle order); particles with non-finite or out-of-box coordinates are
    skipped (``kernels.deposit_rejected``)."""
    dev = _device()
    pos = torch.as_tensor(np.ascontiguousarray(positions, dtype=np.float64), device=dev)
    if pos.ndim != 2 or pos.shape[1] != 3:
        raise ValueError(f"positions must have shape (n, 3), got {tuple(pos.shape)}")
    # a writable copy: a broadcast of an already full-size array is a read-only view
    w = torch.as_tensor(np.array(np.broadcast_to(np.asarray(weights, dtype=np.float64), (pos.shape[0],))),
                        device=dev)
    phi = torch.as_tensor(np.ascontiguousarray(phi_array, dtype=np.float64), device=dev)
    eps, _, _ = kernels.deposit(pos, w, int(J), float(box_size), phi, int(phi_resolution),
                                out_dtype=torch.float64)
    return eps.cpu().numpy()


def interpolate_grid_at_pos_numba(output_values, scaled_positions, grid_values, phi_array, grid_size,
                                  phi_resolution, phi_support, dx=0.0, dy=0.0, dz=0.0):
    """output_values[i] = sum over the 27 stencil points of
    grid[(c - s) & (L - 1)] phi(f + res s) (per axis) at scaled position
    + (dx, dy, dz); fills ``output_values`` in place and returns None, as
    the reference.  The grid is read as float32."""
    if int(phi_support) != 3:
        raise ValueError(f"phi_support={phi_support}: the GPU stencil is 3 points per axis")
    J = _level(grid_size)
    out = np.asarray(output_values)
    dev = _device()
    pos = torch.as_tensor(np.ascontiguousarray(scaled_positions, dtype=np.float64), device=dev)
    if pos.ndim != 2 or pos.shape[1] != 3 or out.shape[0] != pos.shape[0]:
        raise ValueError("scaled_positions must be (n, 3) and output_values (n,)")
    grid = _field_eps(grid_values)
    if grid.numel() != (1 << (3 * J)):
        raise ValueError(f"grid_values has {grid.numel()} cells, grid_size={grid_size}")
    phi = torch.as_tensor(np.ascontiguousarray(phi_array, dtype=np.float64), device=dev)
    res = torch.empty(pos.shape[0], dtype=torch.float64, device=dev)
    from .mc3pcf import _mc_workspace

    ws = _mc_workspace(dev)
    _lib.check(_lib.load().hermes_interp(_ptr(grid), J, _ptr(pos), pos.shape[0], _ptr(phi), phi.numel(),
                                         int(phi_resolution), float(dx), float(dy), float(dz), _ptr(res),
                                         _ptr(ws), ws.numel(), _stream_ptr(dev)), "hermes_interp")
    out[...] = res.cpu().numpy()
    return None


def specialized_convolution_3d(s, w, threads):
    """irfftn(rfftn(s) * w) for a real field s [L, L, L] and an rFFT-grid
    kernel w [L, L, L/2 + 1] (real or complex): float64 [L, L, L]."""
    eps = _field_eps(s)
    L = eps.shape[0]
    J = _level(L)
    kern = torch.as_tensor(np.asarray(w))
    if tuple(kern.shape) != (L, L, L // 2 + 1):
        raise ValueError(f"kernel shape {tuple(kern.shape)} does not match the rFFT grid {(L, L, L // 2 + 1)}")
    dev = eps.device
    if kern.is_complex():
        kr, kc = None, kern.to(device=dev, dtype=torch.complex64).contiguous()
    else:
        kr, kc = kern.to(device=dev, dtype=torch.float32).contiguous(), None
    from .window import rfft_field

    spec = rfft_field(eps)
    sptr = _stream_ptr(dev)
    lib = _lib.load()
    _lib.check(lib.hermes_spectrum_multiply(_ptr(spec), _ptr(kr), _ptr(kc), J, 1.0 / float(L) ** 3, sptr),
               "hermes_spectrum_multiply")
    out = torch.empty_like(eps)
    _lib.check(lib.hermes_fft_c2r(_ptr(spec), _ptr(out), J, sptr), "hermes_fft_c2r")
    return out.double().cpu().numpy()


def _gb300_window(obj, field):
    """This package's WindowFunc for a window object: itself, or one built
    from the reference object's parameters (built-in window types)."""
    from .window import WindowFunc

    if isinstance(obj, WindowFunc):
        return obj
    params = getattr(obj, "window_params", None) or getattr(obj, "input_params", None)
    if not params or getattr(obj, "is_composite_window", False):
        return None
    J, box, phi, res = _field_meta(field)
    if getattr(obj, "phi_array", None) is not None:
        phi = np.asarray(obj.phi_array, dtype=np.float64)
    sfc = {"J": J, "box_size": box, "phi_resolution": res, "phi_array": phi,
           "wavelet_mode": getattr(obj, "wavelet_mode", "db2"), "wavelet_level": getattr(obj, "wavelet_level", 10)}
    keep = ("type", "func", "len_args", "los_args", "other_args", "kernel_mode")
    try:
        return WindowFunc({k: params[k] for k in keep if k in params}, sfc,
                          bandwidth=int(getattr(obj, "bandwidth", 1)))
    except (ValueError, KeyError, TypeError):
        return None


def pair_product_with_window(field1, field2, binning_window_obj, threads):
    """Mean over cells of (field1 convolved with the window) * field2, i.e.
    sum_k eps1_hat K conj(eps2_hat) / L^6 (Parseval), with the k = 0 term in
    float64.  Scalar vertices give the product of mean densities."""
    from .corr2pcf import _is_scalar, field_mean_density
    from .window import materialized_pair_products, pair_products, rfft_field

    if field2 is None:
        field2 = field1
    if _is_scalar(field1) or _is_scalar(field2):
        return field_mean_density(field1) * field_mean_density(field2)
    win = _gb300_window(binning_window_obj, field1)
    e1 = _field_eps(field1)
    e2 = e1 if field2 is field1 else _field_eps(field2)
    L = e1.shape[0]
    if win is not None and win.materialized:
        v, _ = materialized_pair_products([e1, e2], [(0, 1)], [win], exclude_k0=False)
        return float(v[0, 0])
    if win is None or win.is_complex or win.resolved_mode() == "complex_full_fft":
        # any other window: its materialised rFFT-grid kernel
        conv = specialized_convolution_3d(e1, binning_window_obj.as_array(), threads)
        return float(np.einsum("ijk,ijk->", conv, e2.double().cpu().numpy(), optimize=True) / conv.size)
    s1 = rfft_field(e1)
    specs, pair = ([s1], (0, 0)) if e2 is e1 else ([s1, rfft_field(e2)], (0, 1))
    v, k0 = pair_products(specs, [pair], [win], exclude_k0=True)
    dc1 = float(e1.double().sum().item())
    dc2 = dc1 if e2 is e1 else float(e2.double().sum().item())
    return float(v[0, 0] + dc1 * dc2 * k0[0] / float(L) ** 6)


def _radial_bin(bw):
    """A per-sample binning window (parameter dict) as the engine's bin:
    a thin-shell radius, or a BinSpec for the other radial profiles."""
    from .multipole import BinSpec
    from .radial_profiles import SUPPORTED

    if not isinstance(bw, dict):
        bw = getattr(bw, "window_params", None) or getattr(bw, "input_params", None) or {}
    kind = str(bw.get("type", "shell")).strip().lower()
    if kind not in SUPPORTED:
        raise ValueError(f"Unsupported radial profile '{kind}'.")
    la = bw.get("len_args", {}) or {}
    if kind == "shell":
        if la.get("R") is None:
            raise ValueError("shell binning window needs len_args['R']")
        return float(la["R"])
    return BinSpec(kind, la, bw.get("other_args") or None)


def calc_DDD_multipole(deltaD1, deltaD2, deltaD3, binning_window12, binning_window13, l_min, l_max,
                       summation_backend="gb300", gpu_device_id=0, gpu_threads_per_block=(8, 8, 8),
                       cache_multipole_fields=False, cache_dir="", cache_namespace="", threads=1,
                       progress_callback=None, m_progress_callback=None):
    """DDD_l, l = l_min..l_max, for three fields and one (r12, r13) sample:
    returns (l_values int32, ddd_l float64, timing_info).  ``summation_backend``
    'plain' runs the per-sample reference-form contraction on the GPU; any
    other value ('gb300', and the reference's 'gpu' / 'cpu') the batched
    engine.  ``progress_callback`` is called once per l with the reference's
    keyword arguments; ``m_progress_callback`` is not called (the m terms of
    one l are computed together)."""
    from .multipole import MultipoleEngine

    if l_min < 0:
        raise ValueError("l_min must be non-negative.")
    if l_max < 0:
        raise ValueError("l_max must be non-negative.")
    if l_min > l_max:
        raise ValueError("l_min must be less than or equal to l_max.")
    t0 = time.perf_counter()
    J, box, phi, res = _field_meta(deltaD1)
    e1 = _field_eps(deltaD1)
    e2 = _field_eps(deltaD2)
    same23 = deltaD3 is deltaD2
    e3 = e2 if same23 else _field_eps(deltaD3)
    pair = [(_radial_bin(binning_window12), _radial_bin(binning_window13))]
    eng = MultipoleEngine(e1, e2, e3, phi, J, box, res, share23=same23)
    l_values = np.arange(l_min, l_max + 1, dtype=np.int32)
    ddd_l = np.empty(l_values.size, dtype=np.float64)
    rho = deltaD1.field_mean_density(value_unit="grid") if hasattr(deltaD1, "field_mean_density") else None
    if rho is None or np.isclose(rho, 0.0):
        rho = 1.0 / float(1 << (3 * J))
    total_m = sum(l + 1 for l in range(l_min, l_max + 1))
    done_m = 0
    for i, l in enumerate(l_values):
        t_l = time.perf_counter()
        f_s, c_s = eng.timing["fields_s"], eng.timing["contract_s"]
        if summation_backend == "plain":
            ddd_l[i] = eng.ddd_plain(pair, int(l), int(l))[0, 0]
        else:
            ddd_l[i] = eng.ddd(pair, int(l), int(l))[0, 0]
        done_m += int(l) + 1
        if progress_callback is not None:
            progress_callback(l=int(l), l_max=int(l_max), ddd_l=float(ddd_l[i]), zeta_l=float(ddd_l[i] / rho ** 3),
                              elapsed_sec=time.perf_counter() - t_l,
                              conv_elapsed_sec=eng.timing["fields_s"] - f_s,
                              sum_elapsed_sec=eng.timing["contract_s"] - c_s,
                              completed_m_tasks=done_m, total_m_tasks=total_m)
    timing_info = {"conv_elapsed_sec": eng.timing["fields_s"], "sum_elapsed_sec": eng.timing["contract_s"],
                   "sum_h2d_elapsed_sec": 0.0, "sum_kernel_elapsed_sec": eng.timing["contract_s"],
                   "sum_d2h_elapsed_sec": 0.0, "sum_reduce_elapsed_sec": 0.0, "sum_callback_elapsed_sec": 0.0,
                   "total_elapsed_sec": time.perf_counter() - t0}
    return l_values, ddd_l, timing_info


def solve_multipoles_from_ratio(A, B, lmax, rcond_warning=1e12):
    """C_l for A(mu) = B(mu) C(mu): builds the mixing matrix M from B / B_0
    and solves M C = A in float64 on the GPU; returns (C, M, cond(M)) and
    prints the reference's warning when cond(M) > rcond_warning."""
    from .multipole import mixing_solve

    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    if A.shape[0] < lmax + 1 or B.shape[0] < lmax + 1:
        raise ValueError("A and B must have length at least lmax+1.")
    C, M, cond = mixing_solve(A[None, :lmax + 1], B[None, :lmax + 1], int(lmax), device=_device())
    condM = float(cond[0])
    if condM > rcond_warning:
        print(f"[warning] mixing matrix is ill-conditioned: cond(M) = {condM:.3e}")
    return C[0], M[0], condM


def estimate_triplet_product_with_sampled_centers(r12_scaled, r13_scaled, mu, center_scaled, n_rot, sfc_meta,
                                                  sfc_field2, sfc_field3, center="box_random", center_weight=None,
                                                  center_weight_sum=None, seed_base_rot=-1, mu_index=-1, eps1=None,
                                                  rho1=None):
    """Monte Carlo triple product for one mu: the rotated triangles of
    utils/corr3pcf_kernels.py:21-63 (seeded per rotation as the reference)
    around each centre.  box_random: mean of n1 n2 n3 with n1 interpolated
    from eps1; particle: rho1 sum_r sum_i w_i n2 n3 / (n_rot sum_i w_i)
    (rho1 defaults to 1 / L^3)."""
    from .mc3pcf import rotation_offsets, triplet_sum

    L = int(getattr(sfc_meta, "L"))
    J = _level(L)
    phi = torch.as_tensor(np.ascontiguousarray(getattr(sfc_meta, "phi_array"), dtype=np.float64), device=_device())
    if int(getattr(sfc_meta, "phi_support", 3)) != 3:
        raise ValueError("the GPU stencil is 3 points per axis (phi_support=3)")
    centres = np.ascontiguousarray(center_scaled, dtype=np.float64)
    offsets = rotation_offsets(float(r12_scaled), float(r13_scaled), float(mu), int(n_rot), seed_base_rot, mu_index)
    e2, e3 = _field_eps(sfc_field2), _field_eps(sfc_field3)
    if center == "box_random":
        if eps1 is None:
            raise ValueError("eps1 must be provided when center='box_random'.")
        c_t = torch.as_tensor(centres, device=_device())
        s, _ = triplet_sum(_field_eps(eps1), e2, e3, J, c_t, offsets, phi)
        return s / (int(n_rot) * centres.shape[0])
    if center == "particle":
        if rho1 is None:
            rho1 = 1.0 / L ** 3
        if centres.shape[0] == 0:
            return 0.0
        w = np.ones(centres.shape[0]) if center_weight is None else np.asarray(center_weight, dtype=np.float64)
        if w.shape[0] != centres.shape[0]:
            raise ValueError("center_weight must have the same length as center_scaled.")
        wsum = float(np.sum(w)) if center_weight_sum is None else float(center_weight_sum)
        if wsum <= 0.0:
            raise ValueError("Particle-center weights must have a positive sum.")
        c_t = torch.as_tensor(centres, device=_device())
        s, _ = triplet_sum(None, e2, e3, J, c_t, offsets, phi, center_w=w, rho1=1.0)
        return float(rho1) * s / (int(n_rot) * wsum)
    raise ValueError(f"Unknown center='{center}'. Use 'box_random' or 'particle'.")


def _context_array(ctx, host_key, device_key):
    """A context entry as a device tensor: the host array, or the device
    array through __cuda_array_interface__."""
    if ctx.get(host_key) is not None:
        return torch.as_tensor(np.ascontiguousarray(ctx[host_key]), device=_device())
    v = ctx.get(device_key)
    if v is None:
        raise KeyError(f"sum_context has neither '{host_key}' nor '{device_key}'")
    return torch.as_tensor(v, device=_device())


def compute_multipole_m_summand(field_r1_m, field_r2_m, sum_context):
    """One m summand S_m = 4 pi / L^3 sum_x eps1(x) sum_{l1,l2} Gamma3(l1, l2)
    a2(x - l1) a3(x - l2) for the two radial multipole fields of one
    (l, m), by the reference-form GPU contraction; ``sum_context`` is the
    reference's (utils/corr3pcf_multipoles.py:324-390: eps1 as 'data' or
    'data_gpu', Gamma as 'gamma' or 'gamma_gpu', 'L', 'phi_support').
    Returns (complex value, timing dict with the reference's keys)."""
    from .multipole import multipole_contract_plain

    if int(sum_context.get("phi_support", 3)) != 3:
        raise ValueError("the GPU contraction is specialised for a support-3 scaling function")
    t0 = time.perf_counter()
    L = int(sum_context["L"])
    J = _level(L)
    eps1 = _context_array(sum_context, "data", "data_gpu").to(torch.float32).reshape(-1).contiguous()
    gamma = _context_array(sum_context, "gamma", "gamma_gpu").double().cpu().numpy()
    a2 = torch.as_tensor(np.asarray(field_r1_m), device=_device()).to(torch.complex64).reshape(-1).contiguous()
    a3 = torch.as_tensor(np.asarray(field_r2_m), device=_device()).to(torch.complex64).reshape(-1).contiguous()
    if eps1.numel() != L ** 3 or a2.numel() != L ** 3 or a3.numel() != L ** 3:
        raise ValueError("fields and sum_context disagree on the grid size")
    t1 = time.perf_counter()
    value = multipole_contract_plain(eps1, a2, a3, gamma, J)
    t2 = time.perf_counter()
    return value, {"h2d_elapsed_sec": t1 - t0, "kernel_elapsed_sec": t2 - t1, "reduce_elapsed_sec": 0.0,
                   "d2h_elapsed_sec": 0.0}
