"""Radial profiles U_l(k) for multipole windows beyond the thin shell.

Host-side tables for the GPU fields pass (``hermes_multipole_fields_table``),
restating pyhermes/utils/radial_profiles.py:
* real-space profiles w(r) (sphere, thick_shell, gaussian, and user profiles
  from ``real_space_profile`` / ``tabulated_real_space_profile``) are
  integrated by Gauss-Legendre quadrature on their support, normalised to
  4 pi int r^2 w dr = 1 unless their normalisation is "provided" (:182-220,
  :318-360, :421-436);
* k-space transfers (gaussian_shell with R_smooth > 0, and user profiles from
  ``kspace_profile``) are first inverse-Hankel transformed to w(r) on a
  radial quadrature (:362-418);
* U_l(k) = sum_i 4 pi w_i r_i^2 w(r_i) j_l(2 pi k r_i) on a uniform k grid
  over [0, k_max] (:439-446, :651-709); the number of quadrature and table
  points grows with k_max * support exactly as the reference chooses it.
The analytic monopole transfers (l = 0, :222-266) are evaluated on the GPU
directly (``hermes_multipole_fields_window``); thin shells use j_l(2 pi k R).
Lengths and k are physical (box units, cycles per unit length).
"""

import math

import numpy as np
from numpy.polynomial.legendre import leggauss
from scipy.special import spherical_jn

QUAD_MIN, QUAD_PER_CYCLE = 1024, 32
TABLE_MIN, TABLE_PER_CYCLE = 4097, 64
BUILTIN = {"shell", "sphere", "thick_shell", "gaussian", "gaussian_shell"}
CUSTOM = {"custom_real", "custom_kspace"}
SUPPORTED = BUILTIN | CUSTOM
ANALYTIC_MONOPOLE = {"sphere", "thick_shell", "gaussian", "gaussian_shell"}

_GL = {}
_TABLES = {}


def real_space_profile(func, r_max, *, r_min=0.0, normalization="unit_integral", allow_signed=False,
                       quadrature_points=None, table_points=None, args=None):
    """A user real-space profile w(r, **len_args) (utils/radial_profiles.py:39-59)."""
    if not callable(func):
        raise TypeError("real_space_profile requires a callable func(r, **len_args).")
    return {"kind": "real_callable", "func": func, "r_min": float(r_min), "r_max": float(r_max),
            "normalization": str(normalization), "allow_signed": bool(allow_signed),
            "quadrature_points": quadrature_points, "table_points": table_points,
            "args": {} if args is None else dict(args)}


def tabulated_real_space_profile(r, w, *, normalization="unit_integral", allow_signed=False,
                                 quadrature_points=None, table_points=None):
    """A tabulated user real-space profile (utils/radial_profiles.py:62-77)."""
    r = np.asarray(r, dtype=np.float64)
    w = np.asarray(w, dtype=np.float64)
    if r.ndim != 1 or w.ndim != 1 or r.size != w.size or r.size < 2:
        raise ValueError("tabulated_real_space_profile requires matching one-dimensional r and w arrays.")
    return {"kind": "real_tabulated", "r": r, "w": w, "normalization": str(normalization),
            "allow_signed": bool(allow_signed), "quadrature_points": quadrature_points, "table_points": table_points}


def kspace_profile(func, r_max, inverse_k_max, *, r_min=0.0, normalization="unit_integral", allow_signed=True,
                   inverse_points=None, quadrature_points=None, table_points=None, args=None):
    """A user isotropic k-space transfer T(k, **len_args) (utils/radial_profiles.py:80-98)."""
    if not callable(func):
        raise TypeError("kspace_profile requires a callable func(k, **len_args).")
    return {"kind": "kspace_callable", "func": func, "r_min": float(r_min), "r_max": float(r_max),
            "inverse_k_max": float(inverse_k_max), "normalization": str(normalization),
            "allow_signed": bool(allow_signed), "inverse_points": inverse_points,
            "quadrature_points": quadrature_points, "table_points": table_points,
            "args": {} if args is None else dict(args)}


def _length(len_args, name, kind):
    if name not in len_args:
        raise ValueError(f"radial profile '{kind}' requires len_args['{name}'].")
    v = float(len_args[name])
    if not np.isfinite(v):
        raise ValueError(f"radial profile '{kind}' requires finite len_args['{name}'].")
    return v


def _profile_spec(profile_config):
    if profile_config is None:
        raise ValueError("Custom radial profiles require other_args['profile'].")
    if not isinstance(profile_config, dict):
        raise TypeError("Custom radial profile configuration must be a dictionary.")
    spec = dict(profile_config.get("profile", profile_config))
    for key in ("r_min", "r_max", "inverse_k_max", "normalization", "allow_signed", "quadrature_points",
                "inverse_points", "table_points"):
        if key in profile_config:
            spec[key] = profile_config[key]
    return spec


def _point_count(scale, minimum, per_cycle, configured, label):
    if configured is not None:
        n = int(configured)
        if n < 8:
            raise ValueError(f"{label} must be at least 8.")
        return n
    return max(int(minimum), int(math.ceil(per_cycle * max(float(scale), 1.0))) + 1)


def _gauss_legendre(a, b, n):
    if n < 8:
        raise ValueError("Radial Hankel quadrature requires at least 8 points.")
    if n not in _GL:
        _GL[n] = leggauss(n)
    x, w = _GL[n]
    h = 0.5 * (b - a)
    return h * (x + 1.0) + a, h * w


def monopole_transfer(kind, k, len_args):
    """Analytic isotropic transfers U_0(k) (utils/radial_profiles.py:222-266), k physical."""
    k = np.asarray(k, dtype=np.float64)

    def sphere(radius):
        q = 2.0 * np.pi * k * radius
        out = np.ones_like(q)
        nz = q != 0.0
        out[nz] = 3.0 * (np.sin(q[nz]) - q[nz] * np.cos(q[nz])) / q[nz] ** 3
        return out

    if kind == "shell":
        return spherical_jn(0, 2.0 * np.pi * k * _length(len_args, "R", kind))
    if kind == "sphere":
        return sphere(_length(len_args, "R", kind))
    if kind == "thick_shell":
        r, dr = _length(len_args, "R", kind), _length(len_args, "delta_R", kind)
        lo, hi = max(0.0, r - 0.5 * dr), r + 0.5 * dr
        den = hi ** 3 - lo ** 3
        return np.ones_like(k) if den == 0.0 else (hi ** 3 * sphere(hi) - lo ** 3 * sphere(lo)) / den
    if kind == "gaussian":
        q = 2.0 * np.pi * k * _length(len_args, "R", kind)
        return np.exp(-0.5 * q * q)
    if kind == "gaussian_shell":
        r, s = _length(len_args, "R_shell", kind), _length(len_args, "R_smooth", kind)
        den = r * r + s * s
        if den == 0.0:
            return np.ones_like(k)
        qs, qm = 2.0 * np.pi * k * r, 2.0 * np.pi * k * s
        sinc = np.ones_like(qs)
        nz = qs != 0.0
        sinc[nz] = np.sin(qs[nz]) / qs[nz]
        return (s * s * np.cos(qs) + r * r * sinc) / den * np.exp(-0.5 * qm * qm)
    raise ValueError(f"No built-in k-space monopole is available for '{kind}'.")


def _real_profile(kind, len_args, profile_config, k_max):
    """(radii, weights, w(r), options) for real-space profiles."""
    if kind in ("sphere", "thick_shell", "gaussian"):
        if kind == "sphere":
            radius = _length(len_args, "R", kind)
            if radius <= 0.0:
                raise ValueError("sphere radial multipoles require R > 0.")
            lo, hi, opts = 0.0, radius, {"normalization": "provided", "allow_signed": False}

            def func(r):
                return np.where(r <= radius, 3.0 / (4.0 * np.pi * radius ** 3), 0.0)
        elif kind == "thick_shell":
            radius, width = _length(len_args, "R", kind), _length(len_args, "delta_R", kind)
            if width <= 0.0:
                raise ValueError("thick_shell radial multipoles require delta_R > 0.")
            lo, hi = max(0.0, radius - 0.5 * width), radius + 0.5 * width
            vol = 4.0 * np.pi * (hi ** 3 - lo ** 3) / 3.0
            opts = {"normalization": "provided", "allow_signed": False}

            def func(r):
                return np.where((r >= lo) & (r <= hi), 1.0 / vol, 0.0)
        else:
            radius = _length(len_args, "R", kind)
            if radius <= 0.0:
                raise ValueError("gaussian radial multipoles require R > 0.")
            lo, hi = 0.0, 8.0 * radius
            opts = {"normalization": "unit_integral", "allow_signed": False}
            norm = (2.0 * np.pi * radius * radius) ** (-1.5)

            def func(r):
                return norm * np.exp(-0.5 * (r / radius) ** 2)
        if profile_config:
            for key in ("quadrature_points", "inverse_points", "table_points"):
                if key in profile_config:
                    opts[key] = profile_config[key]
        n = _point_count(k_max * (hi - lo), QUAD_MIN, QUAD_PER_CYCLE, opts.get("quadrature_points"),
                         "quadrature_points")
        r, w = _gauss_legendre(lo, hi, n)
        return r, w, func(r), opts
    spec = _profile_spec(profile_config)
    kind2 = str(spec.get("kind", "")).strip().lower()
    if kind2 == "real_tabulated":
        tr, tw = np.asarray(spec["r"], dtype=np.float64), np.asarray(spec["w"], dtype=np.float64)
        if np.any(np.diff(tr) <= 0.0):
            raise ValueError("real_tabulated profile radii must be finite and strictly increasing.")
        lo, hi = float(tr[0]), float(tr[-1])
        n = _point_count(k_max * (hi - lo), max(QUAD_MIN, tr.size), QUAD_PER_CYCLE, spec.get("quadrature_points"),
                         "quadrature_points")
        r, w = _gauss_legendre(lo, hi, n)
        return r, w, np.interp(r, tr, tw), spec
    if kind2 == "real_callable":
        lo, hi = float(spec["r_min"]), float(spec["r_max"])
        n = _point_count(k_max * (hi - lo), QUAD_MIN, QUAD_PER_CYCLE, spec.get("quadrature_points"),
                         "quadrature_points")
        r, w = _gauss_legendre(lo, hi, n)
        kw = dict(spec.get("args", {}))
        kw.update(len_args)
        vals = np.asarray(spec["func"](r, **kw), dtype=np.float64)
        if vals.ndim == 0:
            vals = np.full(r.shape, float(vals))
        if vals.shape != r.shape or not np.all(np.isfinite(vals)):
            raise ValueError("Custom radial profile must return finite values with the same shape as its input.")
        return r, w, vals, spec
    raise ValueError(f"Expected a real-space profile, got kind '{kind2}'.")


def _inverse_profile(kind, len_args, profile_config, k_max):
    """(radii, weights, w(r), options) from a k-space transfer by inverse Hankel."""
    if kind == "gaussian_shell":
        r_shell, smooth = _length(len_args, "R_shell", kind), _length(len_args, "R_smooth", kind)
        if smooth == 0.0:
            raise ValueError("gaussian_shell with R_smooth=0 must use the exact shell path.")
        spec = {"r_min": 0.0, "r_max": r_shell + 8.0 * smooth,
                "inverse_k_max": max(k_max, 8.0 / (2.0 * np.pi * smooth)),
                "normalization": "unit_integral", "allow_signed": True}
        if profile_config:
            for key in ("quadrature_points", "inverse_points", "table_points"):
                if key in profile_config:
                    spec[key] = profile_config[key]

        def transfer(k):
            return monopole_transfer("gaussian_shell", k, len_args)
    else:
        spec = _profile_spec(profile_config)
        if str(spec.get("kind", "")).strip().lower() != "kspace_callable":
            raise ValueError("custom_kspace requires a profile created by kspace_profile.")

        def transfer(k):
            kw = dict(spec.get("args", {}))
            kw.update(len_args)
            return np.asarray(spec["func"](k, **kw), dtype=np.float64)

    lo, hi, kinv = float(spec["r_min"]), float(spec["r_max"]), float(spec["inverse_k_max"])
    nr = _point_count(k_max * (hi - lo), QUAD_MIN, QUAD_PER_CYCLE, spec.get("quadrature_points"), "quadrature_points")
    r, rw = _gauss_legendre(lo, hi, nr)
    nk = _point_count(kinv * hi, QUAD_MIN, QUAD_PER_CYCLE, spec.get("inverse_points"), "inverse_points")
    kn, kw = _gauss_legendre(0.0, kinv, nk)
    pre = 4.0 * np.pi * kw * kn ** 2 * transfer(kn)
    vals = np.empty_like(r)
    for s in range(0, r.size, 64):
        vals[s:s + 64] = spherical_jn(0, 2.0 * np.pi * np.outer(r[s:s + 64], kn)) @ pre
    return r, rw, vals, spec


def _normalise(r, w, vals, opts):
    vals = np.asarray(vals, dtype=np.float64)
    if not np.all(np.isfinite(vals)):
        raise ValueError("Radial profile evaluation produced non-finite values.")
    if not bool(opts.get("allow_signed", False)) and np.any(vals < 0.0):
        raise ValueError("Real-space radial profile has negative values; set allow_signed=True for compensated filters.")
    mode = str(opts.get("normalization", "unit_integral")).strip().lower()
    if mode == "provided":
        return vals
    if mode != "unit_integral":
        raise ValueError("Radial profile normalization must be 'unit_integral' or 'provided'.")
    norm = 4.0 * np.pi * np.sum(w * r ** 2 * vals)
    if not np.isfinite(norm) or np.isclose(norm, 0.0):
        raise ValueError("Radial profile has a non-finite or zero volume integral.")
    return vals / norm


def _freeze(v):
    if callable(v):
        return ("callable", id(v))
    if isinstance(v, np.ndarray):
        return ("array", v.shape, v.tobytes())
    if isinstance(v, dict):
        return tuple(sorted((str(k), _freeze(x)) for k, x in v.items()))
    if isinstance(v, (list, tuple)):
        return tuple(_freeze(x) for x in v)
    return v


def build_radial_multipole_table(radial_type, len_args, l, k_max, profile_config=None):
    """(k_max, U_l on a uniform grid over [0, k_max]) for a non-shell profile
    (utils/radial_profiles.py:651-709)."""
    kind = str(radial_type).strip().lower()
    if kind not in SUPPORTED:
        raise ValueError(f"Unsupported radial profile '{kind}'. Supported profiles: {', '.join(sorted(SUPPORTED))}.")
    if kind == "shell":
        raise ValueError("shell uses the analytic multipole kernel and does not require a radial table.")
    if not np.isfinite(k_max) or k_max <= 0.0:
        raise ValueError("k_max must be finite and positive when tabulating radial multipole windows.")
    key = (kind, _freeze(dict(len_args)), _freeze(profile_config), int(l), float(k_max))
    hit = _TABLES.get(key)
    if hit is not None:
        return hit
    if kind == "gaussian_shell" and float(len_args["R_smooth"]) == 0.0:
        radius = _length(len_args, "R_shell", kind)
        n = _point_count(k_max * radius, TABLE_MIN, TABLE_PER_CYCLE, None, "table_points")
        k = np.linspace(0.0, float(k_max), n)
        out = (float(k_max), np.ascontiguousarray(spherical_jn(int(l), 2.0 * np.pi * k * radius)))
    else:
        if kind in ("sphere", "thick_shell", "gaussian", "custom_real"):
            r, w, vals, opts = _real_profile(kind, len_args, profile_config, k_max)
        else:
            r, w, vals, opts = _inverse_profile(kind, len_args, profile_config, k_max)
        vals = _normalise(r, w, vals, opts)
        n = _point_count(k_max * float(np.max(r)), TABLE_MIN, TABLE_PER_CYCLE, opts.get("table_points"),
                         "table_points")
        k = np.linspace(0.0, float(k_max), n)
        pre = 4.0 * np.pi * w * r ** 2 * vals
        tab = np.empty(n)
        for s in range(0, n, 64):
            tab[s:s + 64] = spherical_jn(int(l), 2.0 * np.pi * np.outer(k[s:s + 64], r)) @ pre
        out = (float(k_max), np.ascontiguousarray(tab))
    if len(_TABLES) > 256:
        _TABLES.pop(next(iter(_TABLES)))
    _TABLES[key] = out
    return out


DIAGNOSTIC_PROBES = 33


def _quadrature(kind, len_args, profile_config, k_max):
    """Normalised (radii, weights, w(r), options) of a tabulated profile."""
    if kind in ("sphere", "thick_shell", "gaussian", "custom_real"):
        r, w, vals, opts = _real_profile(kind, len_args, profile_config, k_max)
    elif kind in ("gaussian_shell", "custom_kspace"):
        r, w, vals, opts = _inverse_profile(kind, len_args, profile_config, k_max)
    else:
        raise ValueError(f"Unsupported tabulated radial profile '{kind}'.")
    return r, w, _normalise(r, w, vals, opts), opts


def _forward_hankel(r, w, vals, l, k):
    """U_l(k) = sum_i 4 pi w_i r_i^2 w(r_i) j_l(2 pi k r_i)."""
    pre = 4.0 * np.pi * w * r ** 2 * vals
    out = np.empty(k.size)
    for s in range(0, k.size, 64):
        out[s:s + 64] = spherical_jn(int(l), 2.0 * np.pi * np.outer(k[s:s + 64], r)) @ pre
    return out


def interpolate_uniform_table(k, table, k_max):
    """The table lookup the GPU kernel makes (utils/radial_profiles.py:
    514-540): linear in the first and last intervals, the four-point local
    cubic (Catmull-Rom form) inside, the last entry at and beyond k_max."""
    k = np.clip(np.asarray(k, dtype=np.float64), 0.0, float(k_max))
    x = k * (table.size - 1) / float(k_max)
    i = np.floor(x).astype(np.intp)
    t = x - i
    top = i >= table.size - 1
    i = np.minimum(i, table.size - 2)
    out = table[i] * (1.0 - t) + table[i + 1] * t
    mid = (i > 0) & (i < table.size - 2)
    if np.any(mid):
        j, u = i[mid], t[mid]
        p0, p1, p2, p3 = table[j - 1], table[j], table[j + 1], table[j + 2]
        out[mid] = 0.5 * (2.0 * p1 + (p2 - p0) * u + (2.0 * p0 - 5.0 * p1 + 4.0 * p2 - p3) * u * u
                          + (3.0 * p1 - p0 - 3.0 * p2 + p3) * u * u * u)
    out[top] = table[-1]
    return out


def diagnose_radial_multipole_table(radial_type, len_args, l, k_max, profile_config=None, *, tolerance=1.0e-5,
                                    probe_count=DIAGNOSTIC_PROBES):
    """Normalisation and convergence of one U_l table
    (utils/radial_profiles.py:559-648): the table at probe_count mid-point
    probes against a transform with doubled quadrature, the k = 0 value
    against 4 pi int r^2 w (l = 0) or 0, and for k-space profiles at l = 0
    the inverse / forward Hankel round trip against the given transfer."""
    kind = str(radial_type).strip().lower()
    if kind not in SUPPORTED:
        raise ValueError(f"Unsupported radial profile '{kind}'. Supported profiles: {', '.join(sorted(SUPPORTED))}.")
    if kind == "shell" or (kind == "gaussian_shell" and float(len_args["R_smooth"]) == 0.0):
        return {"radial_type": kind, "l": int(l), "path": "analytic_shell", "passed": True}
    if not np.isfinite(tolerance) or tolerance <= 0.0:
        raise ValueError("Radial-profile diagnostic tolerance must be finite and positive.")
    probe_count = int(probe_count)
    if probe_count < 3:
        raise ValueError("Radial-profile diagnostics require at least three probe points.")
    table_k_max, table = build_radial_multipole_table(kind, len_args, l, k_max, profile_config)
    r, w, vals, _ = _quadrature(kind, len_args, profile_config, k_max)
    refined = dict(profile_config or {})
    refined["quadrature_points"] = max(2 * int(r.size), 2 * QUAD_MIN)
    if kind in ("gaussian_shell", "custom_kspace"):
        refined["inverse_points"] = refined["quadrature_points"]
    rr, rw, rv, _ = _quadrature(kind, len_args, refined, k_max)
    probe_k = float(k_max) * (np.arange(probe_count, dtype=np.float64) + 0.5) / probe_count
    exact = _forward_hankel(rr, rw, rv, l, probe_k)
    convergence = float(np.max(np.abs(interpolate_uniform_table(probe_k, table, table_k_max) - exact))
                        / max(1.0, float(np.max(np.abs(exact)))))
    zero_target = float(4.0 * np.pi * np.sum(w * r ** 2 * vals)) if int(l) == 0 else 0.0
    zero_mode = float(table[0])
    roundtrip = None
    if kind in ("gaussian_shell", "custom_kspace") and int(l) == 0:
        if kind == "gaussian_shell":
            given = monopole_transfer("gaussian_shell", probe_k, len_args)
        else:
            spec = _profile_spec(profile_config)
            kw = dict(spec.get("args", {}))
            kw.update(len_args)
            given = np.asarray(spec["func"](probe_k, **kw), dtype=np.float64)
            if given.ndim == 0:
                given = np.full(probe_k.shape, float(given))
        back = _forward_hankel(r, w, vals, 0, probe_k)
        roundtrip = float(np.max(np.abs(back - given)) / max(1.0, float(np.max(np.abs(given)))))
    errors = [convergence, abs(zero_mode - zero_target)] + ([roundtrip] if roundtrip is not None else [])
    return {"radial_type": kind, "l": int(l),
            "path": "inverse_hankel" if kind in ("gaussian_shell", "custom_kspace") else "real_space_hankel",
            "table_points": int(table.size), "quadrature_points": int(r.size), "refined_quadrature_points": int(rr.size),
            "probe_count": probe_count, "zero_mode": zero_mode, "zero_mode_target": zero_target,
            "zero_mode_error": float(abs(zero_mode - zero_target)), "table_convergence_error": convergence,
            "inverse_roundtrip_error": roundtrip, "tolerance": float(tolerance), "passed": bool(max(errors) <= tolerance)}


def profile_mode(radial_type, len_args, l):
    """How the GPU evaluates U_l for one bin (radial_multipole_windows.py:
    269-313): 'shell' (j_l(2 pi k R), with R = R_shell for gaussian_shell with
    R_smooth = 0), 'analytic' (l = 0 monopole transfers) or 'table'."""
    kind = str(radial_type).strip().lower()
    if kind == "shell":
        return "shell"
    if kind == "gaussian_shell" and float(len_args.get("R_smooth", 1.0)) == 0.0:
        return "shell"
    if int(l) == 0 and kind in ANALYTIC_MONOPOLE:
        return "analytic"
    return "table"
