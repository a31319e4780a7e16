"""Oracle: float64 CPU restatement of the PyHermes field pipeline.

TEST INFRASTRUCTURE ONLY.  tests/, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` use it as the checker; the product package
(``pyhermes_gb300``) never imports it.

The hot loops live in ``hermes_oracle.c`` (built by ``oracle/build_oracle.py``
into ``oracle/_build/libhermes_oracle.so``); FFTs use scipy.fft (pocketfft),
the same library the reference calls (``pyhermes/utils/convolution.py:7``).
Every function cites the reference lines it restates.
"""

import ctypes
import os

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        from build_oracle import build  # noqa: E402  (sibling module)

        path = build()
        _LIB = ctypes.CDLL(path)
        P = ctypes.c_void_p
        I64 = ctypes.c_int64
        I = ctypes.c_int
        D = ctypes.c_double
        _LIB.oracle_deposit.argtypes = [P, P, I64, P, I, I, I, D, P]
        _LIB.oracle_cell_counts.argtypes = [P, I64, I, D, P]
        _LIB.oracle_interp.argtypes = [P, I64, P, I, P, I, I, D, D, D, P]
        _LIB.oracle_num_threads.restype = I
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def num_threads():
    return int(lib().oracle_num_threads())


def deposit(pos, w, phi, J, box, res=1024):
    """utils/wavelet_grid.py:58-70 project_scaling_grid_numba -> float64 [L,L,L]."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    L = 1 << J
    grid = np.empty((L, L, L), dtype=np.float64)
    lib().oracle_deposit(_p(pos), _p(w), pos.shape[0], _p(phi), phi.size, res, J, float(box), _p(grid))
    return grid


def cell_counts(pos, J, box):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    L = 1 << J
    out = np.empty((L, L, L), dtype=np.uint32)
    lib().oracle_cell_counts(_p(pos), pos.shape[0], J, float(box), _p(out))
    return out


def interp(scaled_pos, grid, phi, J, res=1024, offset=(0.0, 0.0, 0.0)):
    """utils/wavelet_grid.py:143-186 interpolate_grid_at_pos_numba."""
    scaled_pos = np.ascontiguousarray(scaled_pos, dtype=np.float64)
    grid = np.ascontiguousarray(grid, dtype=np.float64)
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    out = np.empty(scaled_pos.shape[0], dtype=np.float64)
    lib().oracle_interp(_p(scaled_pos), scaled_pos.shape[0], _p(grid), J, _p(phi), phi.size, res,
                        float(offset[0]), float(offset[1]), float(offset[2]), _p(out))
    return out


def projection_weights(catalog_weight, field_value, mode="catalog"):
    """base/sfc_projection.py:251-282: float64 p_w = w*q/denominator."""
    cw = np.asarray(catalog_weight, dtype=np.float64)
    fv = np.asarray(field_value, dtype=np.float64)
    cw_sum = float(np.sum(cw, dtype=np.float64))
    raw = float(np.sum(cw * fv, dtype=np.float64))
    if mode == "raw":
        den = 1.0
    elif mode == "catalog":
        den = cw_sum
    else:
        den = raw
    return cw * fv / den, raw / den


WIN_CODES = {
    "sphere": 0, "gaussian": 1, "shell": 2, "thick_shell": 3, "gaussian_shell": 4, "cubic": 5,
    "ring": 6, "disk": 7, "cylshell": 8, "cylinder": 9, "cw": 10, "cws": 11, "gdw": 12,
    "directional_derivative": 13, "laplacian": 14, "inverse_laplacian": 15,
}
WIN_ARGS = {
    "sphere": ("R",), "gaussian": ("R",), "shell": ("R",), "thick_shell": ("R", "delta_R"),
    "gaussian_shell": ("R_shell", "R_smooth"), "cubic": ("Lx", "Ly", "Lz"),
    "ring": ("R", "H"), "disk": ("R", "H"), "cylshell": ("R", "H"), "cylinder": ("R", "H"),
    "cw": ("R",), "cws": ("R",), "gdw": ("R",), "directional_derivative": (),
    "laplacian": (), "inverse_laplacian": (),
}


def fourier_power(phi, k_max, k_count, res=1024):
    """utils/wavelet_grid.py:94-118: |phi_hat|^2 by direct DFT (float64)."""
    phi = np.asarray(phi, dtype=np.float64)
    n = phi.shape[0]
    dx = (n / res) / n
    k = np.arange(k_count + 1) * (k_max / k_count)
    x = np.arange(n) * dx
    arg = (-2 * np.pi * k)[:, None] * x[None, :]
    re = np.sum(phi * dx * np.cos(arg), axis=1)
    im = np.sum(phi * dx * np.sin(arg), axis=1)
    return re ** 2 + im ** 2


def window_kernel(wtype, len_args, L, P, mode="octant", los=(0.0, 0.0, 1.0), bandwidth=1, box=1000.0):
    """The reference WindowFunc kernel (io/window.py:274-332) in float64.

    len_args are physical lengths (rescaled here by L/box like io/window.py:112).
    mode: 'octant' (convolution.py:14-38 + 263-281), 'full_rfft' (:73-157) or
    'complex_rfft' (:168-252).  Returns [L, L, L/2+1] real or complex."""
    args = np.zeros(4)
    for i, nm in enumerate(WIN_ARGS[wtype]):
        args[i] = float(len_args[nm]) * L / box
    los = np.ascontiguousarray(los, dtype=np.float64)
    P = np.ascontiguousarray(P, dtype=np.float64)
    H = L // 2 + 1
    code = WIN_CODES[wtype]
    lb = lib()
    lb.oracle_window_octant.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lb.oracle_window_rfft.argtypes = lb.oracle_window_octant.argtypes
    if mode == "octant":
        out = np.empty((L, L, H), dtype=np.float64)
        lb.oracle_window_octant(code, _p(args), _p(los), L, bandwidth, _p(P), _p(out))
    else:
        out2 = np.empty((L, L, H, 2), dtype=np.float64)
        lb.oracle_window_rfft(code, _p(args), _p(los), L, bandwidth, _p(P), _p(out2))
        out = out2[..., 0] + 1j * out2[..., 1] if mode == "complex_rfft" else out2[..., 0].copy()
    if wtype == "inverse_laplacian":
        out[0, 0, 0] = 0.0
    return out


def convolve(eps, kernel):
    """utils/convolution.py:284-288: irfftn(rfftn(eps) * K)."""
    from scipy.fft import irfftn, rfftn

    sc = rfftn(np.asarray(eps, dtype=np.float64))
    sc *= kernel
    return irfftn(sc, s=eps.shape)


def pair_product(eps1, eps2, kernel):
    """theory/corr2pcf.py:366-372: mean((eps1 conv K) * eps2)."""
    conv = convolve(eps1, kernel)
    return float(np.einsum("ijk,ijk->", conv, eps2, optimize=True) / conv.size)


def cal_gamma(phi, support=3, res=1024):
    """utils/corr3pcf_multipoles.py:22-30."""
    phi = np.asarray(phi, dtype=np.float64)
    g = np.zeros((support, support))
    for a in range(support):
        for b in range(support):
            g[a, b] = np.sum(phi * np.roll(phi, a * res) * np.roll(phi, b * res)) / res
    return g


def _setup_multipole_lib():
    lb = lib()
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lb.oracle_radial_multipole_window.argtypes = [I, P, I, P, I, I, P]
    lb.oracle_contract.argtypes = [P, P, P, P, I, I, ctypes.POINTER(D), ctypes.POINTER(D)]
    lb.oracle_contract_bins.argtypes = [P, P, I, P, I, P, I, P]
    lb.oracle_contract_bins_range.argtypes = [P, P, I, P, I, P, I, I, I, P]
    lb.oracle_contract_range.argtypes = [P, P, P, P, I, I, I, I, ctypes.POINTER(D), ctypes.POINTER(D)]
    lb.oracle_radial_multipole_window_range.argtypes = [I, P, I, P, I, I, I, I, P]
    lb.oracle_spherical_jn.argtypes = [I, D]
    lb.oracle_spherical_jn.restype = D
    lb.oracle_sph_harm.argtypes = [I, I, D, D, D, ctypes.POINTER(D), ctypes.POINTER(D)]
    return lb


RADIAL_CODES = {"shell": 0, "gaussian_shell": 1, "thick_shell": 2, "sphere": 3, "gaussian": 4}


def radial_multipole_window(L, P, radius_grid, l, m, code=0, arg1=0.0):
    """radial_multipole_windows.py:147-183 -> complex128 [L, L, L]."""
    lb = _setup_multipole_lib()
    out = np.empty((L, L, L, 2), dtype=np.float64)
    args = np.array([radius_grid, arg1, 0.0, 0.0])
    P = np.ascontiguousarray(P, dtype=np.float64)
    lb.oracle_radial_multipole_window(L, _p(P), code, _p(args), l, m, _p(out))
    return out[..., 0] + 1j * out[..., 1]


def radial_multipole_window_planes(L, P, radius_grid, l, m, x_begin, x_end, code=0, arg1=0.0):
    """radial_multipole_window on the x planes [x_begin, x_end) only
    (complex128 [x_end - x_begin, L, L]); the per-plane arithmetic is the
    full window's."""
    lb = _setup_multipole_lib()
    out = np.empty((x_end - x_begin, L, L, 2), dtype=np.float64)
    args = np.array([radius_grid, arg1, 0.0, 0.0])
    P = np.ascontiguousarray(P, dtype=np.float64)
    if lb.oracle_radial_multipole_window_range(L, _p(P), code, _p(args), l, m, x_begin, x_end, _p(out)) != 0:
        raise ValueError("bad plane range")
    return out[..., 0] + 1j * out[..., 1]


def contract_planes(data, a2, a3, gamma, x_begin, x_end):
    """compute_3d_summand_cpu (corr3pcf_multipoles.py:134-170) summed over
    the cells of the x planes [x_begin, x_end) only (oracle_contract_range,
    the per-cell arithmetic of contract)."""
    lb = _setup_multipole_lib()
    data = np.ascontiguousarray(data, dtype=np.float64)
    a2 = np.ascontiguousarray(a2, dtype=np.complex128)
    a3 = np.ascontiguousarray(a3, dtype=np.complex128)
    gamma = np.ascontiguousarray(gamma, dtype=np.float64)
    re, im = ctypes.c_double(0.0), ctypes.c_double(0.0)
    if lb.oracle_contract_range(_p(data), _p(a2), _p(a3), _p(gamma), data.shape[0], gamma.shape[0], x_begin, x_end,
                                ctypes.byref(re), ctypes.byref(im)) != 0:
        raise ValueError("bad plane range")
    return complex(re.value, im.value)


def contract(data, a1, a2, gamma):
    """compute_3d_summand_cpu (corr3pcf_multipoles.py:134-170)."""
    lb = _setup_multipole_lib()
    data = np.ascontiguousarray(data, dtype=np.float64)
    a1 = np.ascontiguousarray(a1, dtype=np.complex128)
    a2 = np.ascontiguousarray(a2, dtype=np.complex128)
    gamma = np.ascontiguousarray(gamma, dtype=np.float64)
    re, im = ctypes.c_double(0.0), ctypes.c_double(0.0)
    lb.oracle_contract(_p(data), _p(a1), _p(a2), _p(gamma), data.shape[0], gamma.shape[0],
                       ctypes.byref(re), ctypes.byref(im))
    return complex(re.value, im.value)


def combine_multipole_m_terms(m_values, l):
    """corr3pcf_multipoles.py:173-180."""
    coeff = complex(m_values[0])
    for m in range(1, l + 1):
        coeff += ((-1) ** m) * complex(m_values[m])
        coeff += ((-1) ** (-m)) * np.conj(complex(m_values[m]))
    coeff *= (-1) ** l
    return coeff.real


def multipole_m_summands(eps1, eps2, eps3, R12, R13, l, phi, res=1024, box=1000.0):
    """S_m for m = 0..l at one (r12, r13) (corr3pcf_multipoles.py:505-555);
    R12/R13 physical radii of thin shells."""
    from scipy.fft import fftn, ifftn

    L = eps1.shape[0]
    P = fourier_power(phi, 1, L, res)
    gamma = cal_gamma(phi, phi.shape[0] // res, res)
    s2 = fftn(np.asarray(eps2, dtype=np.float64))
    s3 = fftn(np.asarray(eps3, dtype=np.float64))
    out = []
    for m in range(0, l + 1):
        w2 = radial_multipole_window(L, P, R12 * L / box, l, m)
        w3 = radial_multipole_window(L, P, R13 * L / box, l, -m)
        a2 = ifftn(s2 * w2)
        a3 = ifftn(s3 * w3)
        out.append((4.0 * np.pi) * contract(eps1, a2, a3, gamma) / eps1.size)
    return out


def calc_ddd_multipole(eps1, eps2, eps3, R12, R13, l_min, l_max, phi, res=1024, box=1000.0):
    """calc_DDD_multipole (corr3pcf_multipoles.py:460-579) for thin shells."""
    ddd = []
    for l in range(l_min, l_max + 1):
        ddd.append(combine_multipole_m_terms(multipole_m_summands(eps1, eps2, eps3, R12, R13, l, phi, res, box), l))
    return np.arange(l_min, l_max + 1, dtype=np.int32), np.asarray(ddd)


def contract_bins(data, a2, a3, gamma):
    """S[b2, b3] = contract(data, a2[b2], a3[b3], gamma) for every bin pair in
    one pass (oracle_contract_bins: the same per-pair arithmetic, inner sums
    shared across b2).  a2: [nb2, L, L, L] complex, a3: [nb3, L, L, L]."""
    lb = _setup_multipole_lib()
    data = np.ascontiguousarray(data, dtype=np.float64)
    a2 = np.ascontiguousarray(a2, dtype=np.complex128)
    a3 = np.ascontiguousarray(a3, dtype=np.complex128)
    gamma = np.ascontiguousarray(gamma, dtype=np.float64)
    nb2, nb3 = a2.shape[0], a3.shape[0]
    out = np.zeros((nb2, nb3, 2))
    rc = lb.oracle_contract_bins(_p(data), _p(a2), nb2, _p(a3), nb3, _p(gamma), data.shape[0], _p(out))
    if rc != 0:
        raise ValueError(f"oracle_contract_bins failed ({rc})")
    return out[..., 0] + 1j * out[..., 1]


def multipole_summands_grid(eps1, eps2, eps3, radii12, radii13, l, m, phi, res=1024, box=1000.0, spectra=None):
    """S_m[i, j] for thin shells radii12[i] x radii13[j] (physical) at one
    (l, m): the per-sample step of calc_DDD_multipole
    (corr3pcf_multipoles.py:505-555) for every (r12, r13) pair of the grid,
    each side field built once per radius.  Returns complex [n12, n13]."""
    from scipy.fft import fftn, ifftn

    L = eps1.shape[0]
    P = fourier_power(phi, 1, L, res)
    gamma = cal_gamma(phi, phi.shape[0] // res, res)
    if spectra is None:
        spectra = (fftn(np.asarray(eps2, dtype=np.float64)), fftn(np.asarray(eps3, dtype=np.float64)))
    s2, s3 = spectra
    workers = os.cpu_count() or 1
    a2 = np.stack([ifftn(s2 * radial_multipole_window(L, P, r * L / box, l, m), workers=workers) for r in radii12])
    a3 = np.stack([ifftn(s3 * radial_multipole_window(L, P, r * L / box, l, -m), workers=workers) for r in radii13])
    return (4.0 * np.pi) * contract_bins(eps1, a2, a3, gamma) / eps1.size


def calc_ddd_multipole_grid(eps1, eps2, eps3, radii12, radii13, l_min, l_max, phi, res=1024, box=1000.0):
    """calc_DDD_multipole (corr3pcf_multipoles.py:460-579) for every
    (r12, r13) pair of a thin-shell grid: DDD_l [n12, n13, n_l] and the
    summands S_lm [(l, m >= 0) in order, n12, n13]."""
    from scipy.fft import fftn

    workers = os.cpu_count() or 1
    spectra = (fftn(np.asarray(eps2, dtype=np.float64), workers=workers),
               fftn(np.asarray(eps3, dtype=np.float64), workers=workers))
    ddd = np.zeros((len(radii12), len(radii13), l_max - l_min + 1))
    summands = []
    for li, l in enumerate(range(l_min, l_max + 1)):
        Sm = [multipole_summands_grid(eps1, eps2, eps3, radii12, radii13, l, m, phi, res, box, spectra)
              for m in range(l + 1)]
        summands.extend(Sm)
        for i in range(len(radii12)):
            for j in range(len(radii13)):
                ddd[i, j, li] = combine_multipole_m_terms([S[i, j] for S in Sm], l)
    return ddd, np.asarray(summands)


def legendre_triple_coeff(l, lp, k):
    """special_functions.py:337-363."""
    from scipy.special import gammaln

    s = l + lp + k
    if (k > l + lp) or (k < abs(l - lp)) or (s % 2 != 0):
        return 0.0
    g = s // 2
    log_val = (gammaln(s - 2 * l + 1) + gammaln(s - 2 * lp + 1) + gammaln(s - 2 * k + 1) - gammaln(s + 2)
               + 2 * (gammaln(g + 1) - gammaln(g - l + 1) - gammaln(g - lp + 1) - gammaln(g - k + 1)))
    return float((2 * k + 1) * np.exp(log_val))


def solve_multipoles_from_ratio(A, B, lmax):
    """special_functions.py:366-409 (build_mixing_matrix + solve)."""
    A = np.asarray(A, dtype=np.float64)[:lmax + 1]
    B = np.asarray(B, dtype=np.float64)[:lmax + 1]
    f = B / B[0]
    M = np.zeros((lmax + 1, lmax + 1))
    for l in range(lmax + 1):
        for lp in range(1, lmax + 1):
            if l == lp:
                M[0, l] += f[lp] / (2 * l + 1)
    for k in range(1, lmax + 1):
        for l in range(lmax + 1):
            for lp in range(1, lmax + 1):
                M[k, l] += legendre_triple_coeff(l, lp, k) * f[lp]
    M += np.eye(lmax + 1)
    M *= B[0]
    return np.linalg.solve(M, A), M, np.linalg.cond(M)


def generate_triangle_offsets(R1, R2, mu, phi, costheta1, alpha):
    """utils/corr3pcf_kernels.py:21-63."""
    import math

    st1 = math.sqrt(1.0 - costheta1 * costheta1)
    dx1, dy1, dz1 = st1 * math.cos(phi), st1 * math.sin(phi), costheta1
    if abs(dx1) > 1e-10 or abs(dy1) > 1e-10:
        o1 = [-dy1, dx1, 0.0]
    else:
        o1 = [0.0, -dz1, dy1]
    nr = math.sqrt(o1[0] ** 2 + o1[1] ** 2 + o1[2] ** 2)
    ox1, oy1, oz1 = o1[0] / nr, o1[1] / nr, o1[2] / nr
    ox2, oy2, oz2 = dy1 * oz1 - dz1 * oy1, dz1 * ox1 - dx1 * oz1, dx1 * oy1 - dy1 * ox1
    ca, sa = math.cos(alpha), math.sin(alpha)
    st = math.sqrt(max(0.0, 1.0 - mu * mu))
    dx2 = mu * dx1 + st * (ca * ox1 + sa * ox2)
    dy2 = mu * dy1 + st * (ca * oy1 + sa * oy2)
    dz2 = mu * dz1 + st * (ca * oz1 + sa * oz2)
    return R1 * dx1, R1 * dy1, R1 * dz1, R2 * dx2, R2 * dy2, R2 * dz2


def mc_box_random(eps1, eps2, eps3, J, centers, r12s, r13s, mu, n_rot, seed_base_rot, mu_index, phi):
    """estimate_triplet_product_box_random_centers (corr3pcf_kernels.py:100-140)."""
    n1 = interp(centers, eps1, phi, J)
    total = 0.0
    for irot in range(n_rot):
        np.random.seed(seed_base_rot + irot + mu_index * 1000003)
        a, b, c = np.random.rand(3)
        o = generate_triangle_offsets(r12s, r13s, mu, 2 * np.pi * a, 2.0 * b - 1.0, 2 * np.pi * c)
        n2 = interp(centers, eps2, phi, J, offset=o[0:3])
        n3 = interp(centers, eps3, phi, J, offset=o[3:6])
        total += float(np.sum(n1 * n2 * n3))
    return total / (n_rot * centers.shape[0])


def mlp_forward(params, dims, x):
    """tanh MLP (hidden tanh, linear output) in float64; returns activations."""
    acts, off, h = [], 0, np.asarray(x, dtype=np.float64)
    for l in range(len(dims) - 1):
        K, N = dims[l], dims[l + 1]
        W = params[off:off + K * N].reshape(K, N)
        b = params[off + K * N:off + K * N + N]
        off += K * N + N
        z = h @ W + b
        h = np.tanh(z) if l + 1 < len(dims) - 1 else z
        acts.append(h)
    return acts


def mlp_mse_grad(params, dims, x, t):
    """Mean squared error and its gradient w.r.t. the flat parameters."""
    params = np.asarray(params, dtype=np.float64)
    acts = mlp_forward(params, dims, x)
    y = acts[-1][:, 0]
    n = y.shape[0]
    loss = float(np.mean((y - t) ** 2))
    dy = (2.0 / n) * (y - t)[:, None]
    grads = np.zeros_like(params)
    offs, off = [], 0
    for l in range(len(dims) - 1):
        offs.append(off)
        off += dims[l] * dims[l + 1] + dims[l + 1]
    for l in range(len(dims) - 2, -1, -1):
        K, N = dims[l], dims[l + 1]
        Yl = acts[l]
        dz = dy * (1.0 - Yl ** 2) if l + 1 < len(dims) - 1 else dy
        Xl = np.asarray(x, dtype=np.float64) if l == 0 else acts[l - 1]
        o = offs[l]
        grads[o:o + K * N] = (Xl.T @ dz).ravel()
        grads[o + K * N:o + K * N + N] = dz.sum(axis=0)
        W = params[o:o + K * N].reshape(K, N)
        dy = dz @ W.T
    return loss, grads
