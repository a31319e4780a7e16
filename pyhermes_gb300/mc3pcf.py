"""Monte Carlo 3PCF on the GPU, with an optional learned importance-sampling
proposal for the triangle centres.

``Corr_3PCF`` mirrors ``pyhermes/theory/corr3pcf.py`` (box-random and
particle centres, single process): the same parameters (r12, r13, theta or
mu sampling, n_rot, n_box_centers, base_seed), the same seeds — centres from
``default_rng(base_seed + 1000003)`` in grid units (:1406-1416,
utils/sampling.py:6-10), one ``np.random.seed(base_seed + 1 + irot +
1000003 * mu_index)`` draw of three uniforms per rotation (corr3pcf_kernels.py:
80-86) — the same products (ddd, rrr, delta_ddd, xi12/13/23, zeta, zeta_H, Q)
and the scale_factor**9 rescale.  Triplet sums run in
``hermes_mc_triplets`` (csrc/mc.cu).

``LearnedProposal`` (no reference counterpart): a tanh MLP over
(r12, r13, mu, the density at the centre and the shell-averaged densities at
r12 and r13 around it) trained with the hand-written kernels of csrc/mlp.cu
on uniform-MC triplet samples to predict log E[mbar^2] at a centre, mbar
being the rotation average of f = n1 n2 n3 that the estimator forms.
Centres are then drawn from a pool of uniform candidates with probability
q_i = a/M + (1-a) h_i / sum h, h = exp(prediction / 2) (the variance-optimal
shape sqrt(E mbar^2), mixed with the uniform pool distribution so weights
stay bounded), and each sample is weighted by (1/M)/q_i: the estimator stays
unbiased for the pool mean, hence for the box mean, whatever the network
predicts.  Inference runs on the tensor cores (hermes_mlp_infer_tc).
"""

import ctypes
import logging
import math
import time
import weakref

import numpy as np
import torch

from . import _lib
from .kernels import _ptr, _stream_ptr
from .params import task_params
from .phi import sample_scaling_function
from .sfc_field import (ResultFileIO, SFCField, check_fout, describe_input, normalize_task_weight_normalization,
                        read_numpy_pickle, write_numpy_pickle)
from .window import WindowFunc

logger = logging.getLogger(__name__)
_WS = {}


def _mc_workspace(device):
    key = str(device)
    if key not in _WS:
        n = ctypes.c_size_t(0)
        _lib.check(_lib.load().hermes_mc_workspace_size(ctypes.byref(n)), "mc_workspace_size")
        _WS[key] = torch.empty(n.value, dtype=torch.uint8, device=device)
    return _WS[key]


_BRICKS = {}
_BRICKS_KEEP = 6


def field_bricks(eps, J):
    """The brick-layout copy of a float32 [L^3] field (hermes_field_to_bricks),
    cached per (storage, version, J) so repeated Monte Carlo calls on the same
    field convert it once; the last few are kept."""
    if eps is None:
        return None
    key = (eps.device.type, eps.device.index, eps.data_ptr(), eps._version, int(J))
    hit = _BRICKS.get(key)
    if hit is not None and hit[0]() is eps:
        return hit[1]
    L = 1 << int(J)
    if eps.dtype != torch.float32 or not eps.is_contiguous() or eps.numel() != L ** 3:
        raise ValueError("field_bricks needs a contiguous float32 field of L^3 cells")
    out = torch.empty(L ** 3, dtype=torch.float32, device=eps.device)
    _lib.check(_lib.load().hermes_field_to_bricks(_ptr(eps), int(J), _ptr(out), _stream_ptr(eps.device)),
               "hermes_field_to_bricks")
    if len(_BRICKS) >= _BRICKS_KEEP:
        _BRICKS.pop(next(iter(_BRICKS)))
    _BRICKS[key] = (weakref.ref(eps), out)
    return out


def generate_triangle_offsets(R1, R2, mu, phi, costheta1, alpha):
    """utils/corr3pcf_kernels.py:21-63 (float64, same operation order)."""
    sintheta1 = math.sqrt(1.0 - costheta1 * costheta1)
    dx1 = sintheta1 * math.cos(phi)
    dy1 = sintheta1 * math.sin(phi)
    dz1 = costheta1
    x2, y2, z2 = R1 * dx1, R1 * dy1, R1 * dz1
    if abs(dx1) > 1e-10 or abs(dy1) > 1e-10:
        ox1, oy1, oz1 = -dy1, dx1, 0.0
    else:
        ox1, oy1, oz1 = 0.0, -dz1, dy1
    norm = math.sqrt(ox1 * ox1 + oy1 * oy1 + oz1 * oz1)
    ox1 /= norm
    oy1 /= norm
    oz1 /= norm
    ox2 = dy1 * oz1 - dz1 * oy1
    oy2 = dz1 * ox1 - dx1 * oz1
    oz2 = dx1 * oy1 - dy1 * ox1
    ca, sa = math.cos(alpha), math.sin(alpha)
    st2 = 1.0 - mu * mu
    if st2 < 0.0:
        st2 = 0.0
    st = math.sqrt(st2)
    dx2 = mu * dx1 + st * (ca * ox1 + sa * ox2)
    dy2 = mu * dy1 + st * (ca * oy1 + sa * oy2)
    dz2 = mu * dz1 + st * (ca * oz1 + sa * oz2)
    return x2, y2, z2, R2 * dx2, R2 * dy2, R2 * dz2


def rotation_offsets(R1, R2, mu, n_rot, seed_base_rot=-1, mu_index=-1, rng=None):
    """[n_rot, 6] offsets with the reference's per-rotation seeding (:80-90)."""
    out = np.empty((n_rot, 6))
    two_pi = 2.0 * math.pi
    for irot in range(n_rot):
        if seed_base_rot >= 0:
            seed = seed_base_rot + irot
            if mu_index >= 0:
                seed += mu_index * 1000003
            np.random.seed(seed)
            a, b, c = np.random.rand(3)
        else:
            a, b, c = (rng or np.random).rand(3)
        out[irot] = generate_triangle_offsets(R1, R2, mu, two_pi * a, 2.0 * b - 1.0, two_pi * c)
    return out


def morton_order(centers, L):
    """Permutation putting centres (grid units) in Morton (Z-curve) order of
    their cells, so threads that run together gather nearby cells."""
    c = torch.floor(centers).to(torch.int64) & (L - 1)
    key = torch.zeros(c.shape[0], dtype=torch.int64, device=c.device)
    for bit in range(int(L).bit_length() - 1):
        for ax in range(3):
            key |= ((c[:, ax] >> bit) & 1) << (3 * bit + ax)
    return torch.argsort(key)


def triplet_sum(eps1, eps2, eps3, J, centers, offsets, phi_t, center_w=None, rho1=0.0, samples=False,
                locality=True, bricks=True):
    """sum_i w_i n1_i sum_r n2 n3 (float64) and optionally the per-triplet
    products.  With locality (and no per-triplet output) the centres are put
    in Morton order first: every centre uses the same rotation offsets, so
    neighbouring threads then gather neighbouring cells from L2 (the sum is
    over all centres, so only its rounding order changes).  With bricks the
    gathers read brick-layout copies of the fields (field_bricks; the same
    values bit for bit, fewer DRAM sectors per gather)."""
    dev = eps2.device
    c = torch.as_tensor(np.ascontiguousarray(centers), dtype=torch.float64, device=dev) \
        if not isinstance(centers, torch.Tensor) else centers
    o = torch.as_tensor(np.ascontiguousarray(offsets), dtype=torch.float64, device=dev)
    w = None if center_w is None else torch.as_tensor(center_w, dtype=torch.float64, device=dev)
    if locality and not samples and c.shape[0] > 4096:
        perm = morton_order(c, 1 << J)
        c = c[perm].contiguous()
        if w is not None:
            w = w[perm].contiguous()
    nc, nr = c.shape[0], o.shape[0]
    smp = torch.empty((nc, nr), dtype=torch.float32, device=dev) if samples else None
    ws = _mc_workspace(dev)
    out = ctypes.c_double(0.0)
    lib = _lib.load()
    fn = lib.hermes_mc_triplets
    if bricks:
        eps1, eps2, eps3 = (field_bricks(e, J) for e in (eps1, eps2, eps3))
        fn = lib.hermes_mc_triplets_bricks
    rc = fn(_ptr(eps1), _ptr(eps2), _ptr(eps3), J, _ptr(c), _ptr(w), nc, _ptr(o), nr, _ptr(phi_t), phi_t.numel(),
            phi_t.numel() // 3, float(rho1), ctypes.byref(out), _ptr(smp), _ptr(ws), ws.numel(), _stream_ptr(dev))
    _lib.check(rc, "hermes_mc_triplets")
    return out.value, smp


def interp(grid, J, scaled_pos, phi_t, offset=(0.0, 0.0, 0.0)):
    dev = grid.device
    p = torch.as_tensor(np.ascontiguousarray(scaled_pos), dtype=torch.float64, device=dev) \
        if not isinstance(scaled_pos, torch.Tensor) else scaled_pos
    out = torch.empty(p.shape[0], dtype=torch.float64, device=dev)
    ws = _mc_workspace(dev)
    rc = _lib.load().hermes_interp(_ptr(grid), J, _ptr(p), p.shape[0], _ptr(phi_t), phi_t.numel(),
                                   phi_t.numel() // 3, float(offset[0]), float(offset[1]), float(offset[2]),
                                   _ptr(out), _ptr(ws), ws.numel(), _stream_ptr(dev))
    _lib.check(rc, "hermes_interp")
    return out


def mc_sample(eps1, eps2, eps3, J, pool, phi_t, R1, R2, mu, n, seed=0, idx=None, weights=None, offsets=None,
              bricks=True):
    """(sum f, sum f^2) in float64 over n one-rotation triplets f = w n1 n2 n3
    (hermes_mc_sample): centre pool[idx[k]] (uniform from the pool when idx
    is None), offsets given [n, 6] or drawn on the device for the triangle
    (R1, R2, mu) in grid units."""
    dev = eps2.device
    out = (ctypes.c_double * 2)()
    ws = _mc_workspace(dev)
    lib = _lib.load()
    fn = lib.hermes_mc_sample
    if bricks:
        eps1, eps2, eps3 = (field_bricks(e, J) for e in (eps1, eps2, eps3))
        fn = lib.hermes_mc_sample_bricks
    rc = fn(_ptr(eps1), _ptr(eps2), _ptr(eps3), J, _ptr(pool), pool.shape[0], _ptr(idx), _ptr(weights),
            _ptr(offsets), int(n), float(R1), float(R2), float(mu), int(seed) & ((1 << 64) - 1), _ptr(phi_t),
            phi_t.numel(), phi_t.numel() // 3, out, _ptr(ws), ws.numel(), _stream_ptr(dev))
    _lib.check(rc, "hermes_mc_sample")
    return out[0], out[1]


# product rules per centre mode (theory/corr3pcf.py:30-48)
PRODUCT_DEPS = {"Q": ["zeta", "zeta_H"], "zeta_H": ["xi12", "xi13", "xi23"], "zeta": ["delta_ddd", "rrr"]}
ALLOWED = {"ddd", "rrr", "delta_ddd", "xi12", "xi13", "xi23", "zeta", "zeta_H", "Q"}
PRODUCT_DEPS_PARTICLE = dict(PRODUCT_DEPS, delta_ddd=["d_delta_dd", "r_delta_dd"])
ALLOWED_PARTICLE = ALLOWED | {"d_delta_dd", "r_delta_dd"}


def _centre_arrays(pos, weight, pos_name, weight_name):
    """Explicit particle centres and weights (theory/corr3pcf.py:550-599):
    given together, (N, 3) float64 positions, 1-D weights of length N with a
    positive sum."""
    if (pos is None) != (weight is None):
        raise ValueError(f"{pos_name} and {weight_name} must be provided together for center='particle'. "
                         "This avoids mixing explicit center coordinates with field-derived weights.")
    if pos is None:
        return None, None
    p = np.ascontiguousarray(np.asarray(pos, dtype=np.float64))
    if p.ndim != 2 or p.shape[1] != 3:
        raise ValueError(f"{pos_name} must be an array-like with shape (N, 3), got shape {p.shape}.")
    w = np.ascontiguousarray(np.asarray(weight, dtype=np.float64))
    if w.ndim != 1 or w.shape[0] != p.shape[0]:
        raise ValueError(f"{weight_name} must be a 1D array with length {p.shape[0]}, got shape {w.shape}.")
    if float(np.sum(w)) <= 0.0:
        raise ValueError(f"{weight_name} must have a positive sum.")
    return p, w


class Corr3PCFData(ResultFileIO):
    """Result container (pyhermes/io/corr3pcf.py).  ``save_corr3pcf`` /
    ``load_corr3pcf`` use the reference's NumPy-framed pickle with the same
    top-level keys and order."""

    FILE_KEYS = ("sfc_info1", "sfc_info2", "sfc_info3", "corr3pcf_info", "mu", "theta", "r23", "ddd", "rrr",
                 "d_delta_dd", "r_delta_dd", "delta_ddd", "xi12", "xi13", "xi23", "zeta", "zeta_H", "Q")

    _OWN_SAVE, _OWN_LOAD = "save_corr3pcf", "load_corr3pcf"

    def __init__(self, data_path=None):
        for k in self.FILE_KEYS:
            setattr(self, k, None)
        self.corr3pcf_info = {}
        if data_path:
            self.load_corr3pcf(data_path)

    def save_corr3pcf(self, f_out, overwrite=False):
        f_out = check_fout(self, f_out, overwrite)
        if not f_out:
            return None
        with open(f_out, "wb") as f:
            write_numpy_pickle(f, {k: getattr(self, k) for k in self.FILE_KEYS})
        return f_out

    def load_corr3pcf(self, f_in):
        with open(f_in, "rb") as f:
            d = read_numpy_pickle(f)
        for k in self.FILE_KEYS:
            setattr(self, k, d.get(k))
        self.corr3pcf_info = d.get("corr3pcf_info") or {}


class Corr_3PCF:
    task_name = "Corr_3PCF"

    def __init__(self, param_task=None, device="cuda"):
        self.task_params = task_params(self.task_name, param_task)
        self.device = torch.device(device)
        self.format_params()

    def format_params(self):
        """The task parameters into attributes (theory/corr3pcf.py:154-230); call again after
        editing task_params."""
        tp = self.task_params
        self.sfc_field = tp.get("sfc_field", "")
        for i in (1, 2, 3):
            setattr(self, f"sfc_field{i}", tp.get(f"sfc_field{i}", "") or self.sfc_field)
            r = tp.get(f"random{i}")
            setattr(self, f"random{i}", tp.get("random") if r in (None, "") else r)
        self.weight_normalization = normalize_task_weight_normalization(tp.get("weight_normalization", "catalog"))
        # smoothing windows: a dict needs a 'type' or a 'func'; vertex windows
        # fall back to the shared one (theory/corr3pcf.py:176-183)
        window = tp.get("window")
        self.window = window if (window and (window.get("type") or window.get("func"))) else None
        for i in (1, 2, 3):
            wi = tp.get(f"window{i}")
            wi = wi if (wi and (wi.get("type") or wi.get("func"))) else None
            setattr(self, f"window{i}", wi if wi else (dict(self.window) if self.window else None))
        self.r12, self.r13 = float(tp["r12"]), float(tp["r13"])
        self.n_rot = int(tp["n_rot"])
        self.center = tp["center"]
        if self.center not in ("box_random", "particle"):
            raise ValueError(f"Unknown center='{self.center}'. Use 'box_random' or 'particle'.")
        self.n_box_centers = int(tp["n_box_centers"])
        self.base_seed = int(tp["base_seed"])
        self.particle_pos1 = tp.get("particle_pos1")
        self.particle_weight1 = tp.get("particle_weight1")
        self.random_pos1 = tp.get("random_pos1")
        self.random_weight1 = tp.get("random_weight1")
        self.fout_path = tp.get("fout_path", "")
        allowed, deps = (ALLOWED_PARTICLE, PRODUCT_DEPS_PARTICLE) if self.center == "particle" else (ALLOWED,
                                                                                                    PRODUCT_DEPS)
        prods = tp.get("products", "Q")
        prods = [prods] if isinstance(prods, str) else list(prods)
        self._given_products = list(prods)
        out = []
        for p in prods:
            p = str(p).strip()
            if p not in allowed:
                raise ValueError(f"Unsupported product '{p}' for center='{self.center}'.")
            if p not in out:
                out.append(p)
        i = 0
        while i < len(out):
            for d in deps.get(out[i], []):
                if d not in out:
                    out.append(d)
            i += 1
        self.expanded = out
        ap = str(tp["angle_param"]).strip().lower()
        if ap == "theta":
            t = tp["theta"]
            if isinstance(t, dict):
                self.theta_arr = np.linspace(float(t.get("theta_min", 0.0)), float(t.get("theta_max", math.pi)),
                                             int(t.get("n_theta", 20)))
            else:
                self.theta_arr = np.asarray(t, dtype=np.float64)
            self.mu_arr = np.cos(self.theta_arr)
        elif ap == "mu":
            m = tp["mu"]
            if isinstance(m, dict):
                self.mu_arr = np.linspace(float(m.get("mu_min", -1.0)), float(m.get("mu_max", 1.0)),
                                          int(m.get("n_mu", 20)))
            else:
                self.mu_arr = np.asarray(m, dtype=np.float64)
            self.theta_arr = np.arccos(np.clip(self.mu_arr, -1.0, 1.0))
        else:
            raise ValueError(f"Unsupported angle_param='{tp['angle_param']}'. Use 'theta' or 'mu'.")

    def _field(self, v, what):
        if isinstance(v, SFCField):
            f = v
        elif isinstance(v, str) and v:
            f = SFCField(data_path=v, device=self.device)
        else:
            raise ValueError(f"Missing usable input for {what}.")
        self._density_physical_scale = float(f.scale_factor) ** 3
        if self.weight_normalization == "unit":
            return f.with_normalization("unit")
        if getattr(f, "field_kind", None) != "catalog_field":
            return f.copy()
        return f.switch_weight_normalization(self.weight_normalization)

    def _windowed(self, i, field):
        """A vertex field after its smoothing window, or a copy
        (theory/corr3pcf.py:463-476, :1038-1050)."""
        w = getattr(self, f"window{i}")
        if w is None:
            return field
        if self.center == "particle" and i == 1:
            # vertex 1 is the particle centres themselves (theory/corr3pcf.py:836-839)
            logger.warning("window1 has no effect for center='particle'; vertex 1 uses particle centres directly.")
            return field
        if isinstance(w, WindowFunc):
            return field @ w
        if isinstance(w, dict):
            return field @ WindowFunc(w, field.sfc_info, device=self.device)
        raise ValueError(f"Unsupported window input for vertex {i}. Expected dict, WindowFunc, or None, "
                         f"got {type(w)}.")

    def _rand(self, i, ref):
        """A uniform random is the mean density of the vertex's windowed data
        field (theory/corr3pcf.py:1076-1091); a random field gets the
        vertex's window."""
        r = getattr(self, f"random{i}")
        if r == "uniform":
            return float(ref.field_mean_density(value_unit="grid"))
        if r is None or r == "":
            return None
        return self._windowed(i, self._field(r, f"random vertex {i}"))

    @staticmethod
    def _density(x):
        return float(x) if isinstance(x, float) else float(x.field_mean_density(value_unit="grid"))

    def _pair(self, radius, a, b):
        """corr3pcf.py:730-734 via the Parseval pair-product engine (shell window)."""
        if isinstance(a, float) or isinstance(b, float):
            return self._density(a) * self._density(b)
        from .corr2pcf import Corr_2PCF

        t = Corr_2PCF({"Corr_2PCF": {"sfc_field1": a, "sfc_field2": b, "weight_normalization": "raw",
                                     "binning_window": {"type": "shell", "len_args": ["R"], "mapping": "s_to_R"},
                                     "sampling": {"s": np.atleast_1d(radius)}, "products": ["dd"]}},
                      device=self.device)
        t._field_in_task_normalization = lambda f: f
        t.prepare_input_fields()
        t._density_physical_scale = 1.0
        return np.asarray(t.run(save_result=False).dd)

    def calc_pair_product(self, radius, field1, field2):
        """theory/corr3pcf.py:730-734: the thin-shell pair product at radius
        (a scalar vertex gives the product of mean densities)."""
        return self._pair(radius, field1, field2)

    def run(self, save_result=True, overwrite=False):
        data = {i: self._windowed(i, self._field(getattr(self, f"sfc_field{i}"), f"field vertex {i}"))
                for i in (1, 2, 3)}
        ref = data[1]
        rand = {i: self._rand(i, data[i]) for i in (1, 2, 3)}
        L, J = ref.L, ref.J
        phi = ref.sfc_info.get("phi_array")
        if phi is None:
            phi = sample_scaling_function(ref.wavelet_mode, ref.wavelet_level)
        phi_t = torch.as_tensor(np.asarray(phi, dtype=np.float64), device=self.device)
        sf = float(ref.scale_factor)
        r12s, r13s = self.r12 * sf, self.r13 * sf
        eps = {i: data[i].epsilon_device.to(torch.float32).contiguous() for i in (1, 2, 3)}

        def delta(i):
            r = rand[i]
            if isinstance(r, float):
                return (data[i].epsilon_device.double() - r).float().contiguous()
            return (data[i].epsilon_device.double() - r.epsilon_device.double()).float().contiguous()

        seed_base_rot = self.base_seed + 1
        n = self.mu_arr.size

        def mc(prod_fields, c_t, w_c, norm):
            """sum over rotations and centres for every mu, divided by norm."""
            e1, e2, e3 = prod_fields
            vals = np.zeros(n)
            for it, mu in enumerate(self.mu_arr):
                off = rotation_offsets(r12s, r13s, float(mu), self.n_rot, seed_base_rot, it)
                s, _ = triplet_sum(e1, e2, e3, J, c_t, off, phi_t, center_w=w_c, rho1=1.0)
                vals[it] = s / norm
            return vals

        res = {}
        if self.center == "box_random":
            rng = np.random.default_rng(self.base_seed + 1000003 * 1)
            centers = rng.uniform(0.0, float(L), size=(self.n_box_centers, 3))
            c_t = torch.as_tensor(centers, dtype=torch.float64, device=self.device)
            norm = float(self.n_rot * centers.shape[0])
            if "ddd" in self.expanded:
                res["ddd"] = mc((eps[1], eps[2], eps[3]), c_t, None, norm)
            if "delta_ddd" in self.expanded:
                res["delta_ddd"] = mc((delta(1), delta(2), delta(3)), c_t, None, norm)
            rho1_rrr = None
        else:
            # particle centres (theory/corr3pcf.py:1134-1180, 1425-1450): n1 is
            # rho1 = (sum of the centre weights) / V, so each estimate is
            # rho1 sum_r sum_i w_i n2 n3 / (n_rot sum_i w_i); r_delta_dd uses
            # the random centres (or the data centres when none are given)
            cpos, cw = _centre_arrays(self.particle_pos1, self.particle_weight1, "particle_pos1", "particle_weight1")
            rpos, rw = _centre_arrays(self.random_pos1, self.random_weight1, "random_pos1", "random_weight1")
            # without explicit centres: the catalogues behind vertex 1's data
            # and random fields, weighted by their projection weights
            # (theory/corr3pcf.py:578-613, 815-833)
            if cpos is None and any(p in self.expanded for p in ("ddd", "d_delta_dd")):
                pd = data[1].get_particle_data()
                cpos, cw = _centre_arrays(pd["pos"], pd["projection_weight"], "sfc_field1 particle positions",
                                          "sfc_field1 particle weight")
            if rpos is None and "r_delta_dd" in self.expanded and isinstance(rand[1], SFCField):
                pd = rand[1].get_particle_data()
                rpos, rw = _centre_arrays(pd["pos"], pd["projection_weight"], "random1 particle positions",
                                          "random1 particle weight")
            V = float(L) ** 3
            rho1_rrr = None
            if cpos is not None:
                wsum = float(cw.sum())
                rho1_p = wsum / V
                c_t = torch.as_tensor(cpos * sf, dtype=torch.float64, device=self.device)
                rho1_rrr = rho1_p
            if rpos is not None:
                rwsum = float(rw.sum())
                rho1_rrr = rwsum / V
                r_t = torch.as_tensor(rpos * sf, dtype=torch.float64, device=self.device)
            needs_data_centres = any(p in self.expanded for p in ("ddd", "d_delta_dd")) or \
                ("r_delta_dd" in self.expanded and rpos is None and not isinstance(rand[1], float))
            if needs_data_centres and cpos is None:
                raise ValueError("center='particle' needs particle_pos1 and particle_weight1, or a catalog "
                                 "sfc_field1 whose particles can be re-read.")
            if "ddd" in self.expanded:
                res["ddd"] = rho1_p * mc((None, eps[2], eps[3]), c_t, cw, self.n_rot * wsum)
            if "d_delta_dd" in self.expanded:
                res["d_delta_dd"] = rho1_p * mc((None, delta(2), delta(3)), c_t, cw, self.n_rot * wsum)
            if "r_delta_dd" in self.expanded and not (rpos is None and isinstance(rand[1], float)):
                if rpos is not None:
                    res["r_delta_dd"] = rho1_rrr * mc((None, delta(2), delta(3)), r_t, rw, self.n_rot * rwsum)
                else:
                    res["r_delta_dd"] = rho1_p * mc((None, delta(2), delta(3)), c_t, cw, self.n_rot * wsum)
        shortcut_r = (self.center == "particle" and "r_delta_dd" in self.expanded and "r_delta_dd" not in res)
        r23 = np.sqrt(np.clip(self.r12 ** 2 + self.r13 ** 2 - 2 * self.r12 * self.r13 * self.mu_arr, 0, None))
        if "rrr" in self.expanded or shortcut_r:
            # theory/corr3pcf.py:736-772 (_compute_rrr_value) and 1346-1351,
            # 1597-1602 (rrr deferred to rho1 RR23 when xi23 is requested with a
            # uniform random vertex 1 and no random centres)
            uniform = [isinstance(rand[i], float) for i in (1, 2, 3)]
            deferred = "xi23" in self.expanded and uniform[0] and self.random_pos1 is None
            r1 = rho1_rrr if (self.center == "particle" and not deferred and rho1_rrr is not None) else None
            if sum(uniform) >= 2 or uniform[0]:
                r1 = self._density(rand[1]) if r1 is None else r1
            if sum(uniform) >= 2:
                rrr = np.full(n, r1 * self._density(rand[2]) * self._density(rand[3]))
            elif uniform[0]:
                rrr = r1 * np.asarray(self._pair(r23, rand[2], rand[3]), dtype=np.float64).reshape(n)
            elif uniform[1]:
                rrr = np.full(n, self._density(rand[2]) * float(np.asarray(self._pair(self.r13, rand[1], rand[3]))[0]))
            elif uniform[2]:
                rrr = np.full(n, self._density(rand[3]) * float(np.asarray(self._pair(self.r12, rand[1], rand[2]))[0]))
            else:  # three random fields: Monte Carlo over the same centres and rotations
                if any(rand[i] is None for i in (1, 2, 3)):
                    raise ValueError("rrr needs random1, random2 and random3 (or 'uniform').")
                reps = {i: rand[i].epsilon_device.to(torch.float32).contiguous() for i in (1, 2, 3)}
                if self.center == "box_random":
                    rrr = mc((reps[1], reps[2], reps[3]), c_t, None, norm)
                else:
                    rt, rwt, rws = (r_t, rw, rwsum) if rpos is not None else (c_t, cw, wsum)
                    r1 = rho1_rrr if rho1_rrr is not None else self._density(rand[1])
                    rrr = r1 * mc((None, reps[2], reps[3]), rt, rwt, self.n_rot * rws)
            res["rrr"] = rrr
        scale = float(getattr(self, "_density_physical_scale", 1.0)) ** 3
        for p in ("ddd", "rrr", "d_delta_dd", "r_delta_dd", "delta_ddd"):
            if p in res:
                res[p] = res[p] * scale
        out = Corr3PCFData()
        out.mu, out.theta = self.mu_arr, self.theta_arr
        out.r23 = np.sqrt(np.clip(self.r12 ** 2 + self.r13 ** 2 - 2 * self.r12 * self.r13 * self.mu_arr, 0, None))
        for p in ("ddd", "rrr", "d_delta_dd", "r_delta_dd", "delta_ddd"):
            setattr(out, p, res.get(p))
        if "xi12" in self.expanded:
            out.xi12 = self._xi(self.r12, data[1], data[2], rand[1], rand[2])
        if "xi13" in self.expanded:
            out.xi13 = self._xi(self.r13, data[1], data[3], rand[1], rand[3])
        if "xi23" in self.expanded or "rrr" in self.expanded or shortcut_r:  # corr3pcf.py:1207 pair cache
            out.xi23 = self._xi(out.r23, data[2], data[3], rand[2], rand[3])
        if shortcut_r:  # uniform random vertex 1 without random centres: r_delta_dd = rrr xi23
            out.r_delta_dd = out.rrr * out.xi23
        if self.center == "particle" and "delta_ddd" in self.expanded:
            out.delta_ddd = out.d_delta_dd - out.r_delta_dd
        if "zeta" in self.expanded:
            out.zeta = out.delta_ddd / out.rrr
        if "zeta_H" in self.expanded:
            out.zeta_H = out.xi12 * out.xi13 + out.xi12 * out.xi23 + out.xi13 * out.xi23
        if "Q" in self.expanded:
            out.Q = out.zeta / out.zeta_H
        for i in (1, 2, 3):
            setattr(out, f"sfc_info{i}", data[i].sfc_info)
        out.corr3pcf_info = self._info_snapshot(rand)
        self.corr3pcf_data = out
        if save_result and self.fout_path:
            out.save_corr3pcf(self.fout_path, overwrite=overwrite)
        return out

    def _info_snapshot(self, rand):
        """corr3pcf_info with the reference's keys (theory/corr3pcf.py:330-380)."""
        def arr(name):
            v = getattr(self, name)
            return None if v is None else {"kind": name, "shape": tuple(np.asarray(v).shape)}

        tp = self.task_params
        info = {"sfc_field": describe_input(self.sfc_field)}
        for i in (1, 2, 3):
            info[f"sfc_field{i}"] = describe_input(getattr(self, f"sfc_field{i}"))
        info.update({"particle_pos1": arr("particle_pos1"), "particle_weight1": arr("particle_weight1"),
                     "random": describe_input(tp.get("random"))})
        for i in (1, 2, 3):
            info[f"random{i}"] = describe_input(rand.get(i))
        info.update({"random_pos1": arr("random_pos1"), "random_weight1": arr("random_weight1"),
                     "weight_normalization": self.weight_normalization, "window": describe_input(self.window)})
        for i in (1, 2, 3):
            info[f"window{i}"] = describe_input(getattr(self, f"window{i}"))
        theta, mu = tp.get("theta"), tp.get("mu")
        info.update({"r12": self.r12, "r13": self.r13, "angle_param": str(tp["angle_param"]).strip().lower(),
                     "theta_spec": describe_input(theta), "mu_spec": describe_input(mu),
                     "n_theta": int(self.theta_arr.size), "n_mu": int(self.mu_arr.size),
                     "theta_min": float(self.theta_arr.min()), "theta_max": float(self.theta_arr.max()),
                     "mu_min": float(self.mu_arr.min()), "mu_max": float(self.mu_arr.max()), "n_rot": self.n_rot,
                     "center": self.center, "n_box_centers": self.n_box_centers, "base_seed": self.base_seed,
                     "threads": int(tp.get("threads", 1)), "products": self._given_products,
                     "fout_path": self.fout_path})
        return info

    def _xi(self, radius, fa, fb, ra, rb):
        """corr3pcf.py:1011-1036: xi = delta_dd / rr with shell pair products."""
        rr = self._pair(radius, ra, rb)
        da = fa - (ra if isinstance(ra, float) else ra)
        db = fb - (rb if isinstance(rb, float) else rb)
        dd = self._pair(radius, da, db)
        return np.asarray(dd) / np.asarray(rr)


# ---------------------------------------------------------------------------
# learned proposal
# ---------------------------------------------------------------------------
class MLP:
    """tanh MLP trained and run with the kernels of csrc/mlp.cu."""

    def __init__(self, dims=(4, 128, 128, 128, 1), device="cuda", seed=0):
        self.dims = list(dims)
        self.device = torch.device(device)
        self.cdims = (ctypes.c_int32 * len(self.dims))(*self.dims)
        n = ctypes.c_int64(0)
        _lib.check(_lib.load().hermes_mlp_param_count(self.cdims, len(self.dims) - 1, ctypes.byref(n)),
                   "mlp_param_count")
        self.n_params = n.value
        g = torch.Generator().manual_seed(seed)
        parts = []
        for a, b in zip(self.dims[:-1], self.dims[1:]):
            parts.append((torch.randn(a, b, generator=g) * math.sqrt(1.0 / a)).reshape(-1))
            parts.append(torch.zeros(b))
        self.params = torch.cat(parts).to(self.device, torch.float32).contiguous()
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step_count = 0
        self.params_bf16 = None

    def _acts(self, batch):
        return torch.empty(sum(batch * d for d in self.dims[1:]), dtype=torch.float32, device=self.device)

    def forward(self, x, bf16=False, return_acts=False):
        x = x.to(torch.float32).contiguous()
        acts = self._acts(x.shape[0])
        lib = _lib.load()
        if bf16:
            if self.params_bf16 is None:
                self.params_bf16 = torch.empty(self.n_params, dtype=torch.bfloat16, device=self.device)
                _lib.check(lib.hermes_to_bf16(_ptr(self.params), self.n_params, _ptr(self.params_bf16),
                                              _stream_ptr(self.device)), "to_bf16")
            rc = lib.hermes_mlp_forward(None, _ptr(self.params_bf16), self.cdims, len(self.dims) - 1, _ptr(x),
                                        x.shape[0], _ptr(acts), _stream_ptr(self.device))
        else:
            rc = lib.hermes_mlp_forward(_ptr(self.params), None, self.cdims, len(self.dims) - 1, _ptr(x), x.shape[0],
                                        _ptr(acts), _stream_ptr(self.device))
        _lib.check(rc, "hermes_mlp_forward")
        y = acts[-x.shape[0] * self.dims[-1]:].view(x.shape[0], self.dims[-1])
        return (y, acts) if return_acts else y

    def infer(self, x):
        """Outputs [batch] with the 128 x 128 hidden layers on the tensor
        cores (hermes_mlp_infer_tc; BF16 weights and activations)."""
        x = x.to(torch.float32).contiguous()
        y = torch.empty(x.shape[0], dtype=torch.float32, device=self.device)
        st = torch.zeros(1, dtype=torch.int32, device=self.device)
        _lib.check(_lib.load().hermes_mlp_infer_tc(_ptr(self.params), self.cdims, len(self.dims) - 1, _ptr(x),
                                                   x.shape[0], _ptr(y), _ptr(st), _stream_ptr(self.device)),
                   "hermes_mlp_infer_tc")
        return y

    def grads(self, x, target, loss="mse", offset=None):
        """(loss, gradient) for one batch: the mean squared error, or
        loss='poisson' the Poisson deviance of log-mean outputs.  `offset`
        (per sample) is added to the output before the loss, a known term
        of the log-mean that the network does not have to learn; the
        gradient with respect to the output is unchanged by it."""
        lib = _lib.load()
        x = x.to(torch.float32).contiguous()
        y, acts = self.forward(x, return_acts=True)
        yv = y.reshape(-1)
        if offset is not None:
            yv = yv + offset.to(torch.float32).reshape(-1)
        yv = yv.contiguous()
        t = target.to(torch.float32).reshape(-1).contiguous()
        dy = torch.empty_like(t)
        scratch_d = torch.empty(1, dtype=torch.float64, device=self.device)
        fn = lib.hermes_poisson_grad if loss == "poisson" else lib.hermes_mse_grad
        lv = ctypes.c_double(0.0)
        _lib.check(fn(_ptr(yv), _ptr(t), t.numel(), _ptr(dy), ctypes.byref(lv), _ptr(scratch_d),
                      _stream_ptr(self.device)), "loss_grad")
        n = ctypes.c_int64(0)
        lib.hermes_mlp_scratch_floats(x.shape[0], ctypes.byref(n))
        scratch = torch.empty(n.value, dtype=torch.float32, device=self.device)
        g = torch.empty_like(self.params)
        _lib.check(lib.hermes_mlp_backward(_ptr(self.params), self.cdims, len(self.dims) - 1, _ptr(x), x.shape[0],
                                           _ptr(acts), _ptr(dy), _ptr(g), _ptr(scratch), _stream_ptr(self.device)),
                   "mlp_backward")
        return lv.value, g

    def adam(self, g, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        self.params_bf16 = None
        _lib.check(_lib.load().hermes_adam_step(_ptr(self.params), _ptr(g), _ptr(self.m), _ptr(self.v),
                                                self.n_params, lr, b1, b2, eps, self.step_count,
                                                _stream_ptr(self.device)), "adam_step")

    def train(self, x, t, epochs=5, batch=8192, lr=2e-3, seed=0, loss="mse", offset=None):
        n = x.shape[0]
        gen = torch.Generator(device=self.device).manual_seed(seed)
        losses = []
        for _ in range(epochs):
            perm = torch.randperm(n, device=self.device, generator=gen)
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                loss_v, g = self.grads(x[idx], t[idx], loss=loss, offset=None if offset is None else offset[idx])
                self.adam(g, lr=lr)
                losses.append(loss_v)
        return losses


class LearnedProposal:
    """Importance sampling of triangle centres with a trained MLP proposal.

    The per-centre value of the reference estimator is a rotation average
    g(c) = n1(c) * mean_r n2 n3, so its second moment given the centre is
    E[g^2 | c] = n1(c)^2 * E[(mean_r n2 n3)^2 | c].  The first factor is known
    exactly at every candidate (the same 27-point interpolation the triplet
    kernel uses), so the proposal keeps it as a fixed factor and the network
    learns only the second: log E[(mean_r n2 n3)^2 | c] as a Poisson-deviance
    fit with log n1^2 as an offset.  Its features are the triangle's shape,
    log n1, and the densities of vertices 2 and 3 averaged over the thin
    shells of radius r12 and r13 around c (the fields convolved with a shell
    window, evaluated with the same interpolation).  Centres with n1 = 0
    contribute exactly 0 to the estimate, so they get no samples; the
    defensive mixture is uniform over the others.  The variance-optimal
    proposal for a weighted mean of per-centre rotation averages is
    q ~ sqrt(E[g^2 | c]), which is what is sampled."""

    N_FEATURES = 6

    def __init__(self, eps1, eps2, eps3, J, phi, rho, device="cuda", mix=0.1):
        self.e1, self.e2, self.e3 = (e.to(torch.float32).contiguous() for e in (eps1, eps2, eps3))
        self.J, self.L = J, 1 << J
        self.phi_np = np.asarray(phi, dtype=np.float64)
        self.phi_t = torch.as_tensor(self.phi_np, device=device)
        self.rho = float(rho)
        self.device = torch.device(device)
        self.mix = mix
        self.net = MLP(dims=(self.N_FEATURES, 128, 128, 128, 1), device=device)
        self._shells = {}

    def shell_field(self, vertex, radius):
        """Field of vertex 2 or 3 averaged over a thin shell of `radius`
        (grid units) around every cell: field @ shell window (W(0) = 1)."""
        src = self.e2 if vertex == 2 else self.e3
        key = (src.data_ptr(), round(float(radius), 6))
        f = self._shells.get(key)
        if f is None:
            from .window import WindowFunc, apply_window

            w = WindowFunc({"type": "shell", "len_args": {"R": float(radius)}},
                           {"J": self.J, "box_size": float(self.L), "phi_resolution": 1024, "wavelet_mode": "db2",
                            "wavelet_level": 10, "phi_array": self.phi_np}, device=self.device)
            f = apply_window(src, w)
            self._shells[key] = f
        return f

    # densities enter on a log scale clamped to [1e-2, 1e3] times the mean
    # density: centres with nothing in reach must not dominate the inputs
    LOG_FLOOR, LOG_CEIL = 1e-2, 1e3

    def _logd(self, v, power=1):
        return torch.log((v / self.rho ** power).clamp(self.LOG_FLOOR, self.LOG_CEIL ** power))

    def features(self, centers, r12s, r13s, mu, return_n1=False):
        """[n, 6] float32 network inputs; with return_n1 also the float64
        centre density n1 (in units of the mean density)."""
        n1 = interp(self.e1, self.J, centers, self.phi_t)
        s2 = interp(self.shell_field(2, r12s), self.J, centers, self.phi_t)
        s3 = interp(self.shell_field(3, r13s), self.J, centers, self.phi_t)
        f = torch.stack([torch.full_like(n1, r12s / self.L * 10), torch.full_like(n1, r13s / self.L * 10),
                         torch.full_like(n1, mu), self._logd(n1), self._logd(s2), self._logd(s3)], dim=1).float()
        return (f, n1.double() / self.rho) if return_n1 else f

    def training_data(self, configs, n_centers, n_rot_train, seed=0, n_rot_eval=100):
        """Uniform-MC samples at centres with n1 != 0: features, the offset
        log n1^2 and, per centre, an unbiased estimate of E[g^2 | centre]
        for the rotation average g of an estimator that uses n_rot_eval
        rotations per centre: from the n_rot_train rotations' mean m and
        variance s^2 (f = n1 n2 n3 in units of the cubed mean density),
        m^2 - (1/n_rot_train - 1/n_rot_eval) s^2, clamped at 0."""
        X, T, O = [], [], []
        rng = np.random.default_rng(seed)
        k = 1.0 / n_rot_train - 1.0 / n_rot_eval
        for (r12s, r13s, mu) in configs:
            c = torch.as_tensor(rng.uniform(0.0, float(self.L), (n_centers, 3)), device=self.device)
            feats, n1 = self.features(c, r12s, r13s, mu, return_n1=True)
            keep = n1 != 0.0
            c, feats, n1 = c[keep].contiguous(), feats[keep], n1[keep]
            off = rotation_offsets(r12s, r13s, mu, n_rot_train, rng=np.random.RandomState(rng.integers(1 << 31)))
            _, smp = triplet_sum(self.e1, self.e2, self.e3, self.J, c, off, self.phi_t, samples=True)
            f = smp.double() / self.rho ** 3
            m, v = f.mean(dim=1), f.var(dim=1)
            X.append(feats)
            T.append((m * m - k * v).clamp_min(0.0))
            O.append(torch.log(n1 * n1))
        return torch.cat(X), torch.cat(T), torch.cat(O)

    def train(self, configs, n_centers=200_000, n_rot_train=8, epochs=4, seed=0, n_rot_eval=100):
        """Fits log E[g^2 | centre] - log n1^2 (targets in units of their
        mean) with the Poisson deviance, whose minimiser is the log of the
        conditional mean even though each target is a noisy few-rotation
        estimate."""
        X, T, O = self.training_data(configs, n_centers, n_rot_train, seed, n_rot_eval)
        self.t_scale = float(T.mean()) or 1.0
        t = (T / self.t_scale).clamp_max(1.0e4).float()
        return self.net.train(X, t, epochs=epochs, seed=seed, loss="poisson", offset=O.float())

    def proposal(self, pool, r12s, r13s, mu, bf16=True):
        """q over the pool: mix uniform over the candidates with n1 != 0 plus
        (1 - mix) |n1| sqrt(exp(network)), normalised; bf16=True evaluates
        the network on the tensor cores (hermes_mlp_infer_tc), False in FP32
        on the CUDA cores."""
        feats, n1 = self.features(pool, r12s, r13s, mu, return_n1=True)
        pred = (self.net.infer(feats) if bf16 else self.net.forward(feats)).reshape(-1).double()
        p = 0.5 * pred.clamp(-60.0, 60.0)  # log sqrt(E[g^2 | centre] / n1^2), relative
        h = n1.abs() * torch.exp(p - p.max())
        support = (n1 != 0.0).double()
        n_sup = float(support.sum())
        if n_sup == 0.0:  # every candidate contributes 0
            return torch.full_like(h, 1.0 / pool.shape[0])
        return self.mix * support / n_sup + (1.0 - self.mix) * h / h.sum()

    def estimate(self, pool, r12s, r13s, mu, n_samples, seed=0, uniform=False, bf16=True):
        """Mean over the pool of E_rot[f]: returns (estimate, per-sample values)."""
        gen = torch.Generator(device=self.device).manual_seed(seed)
        M = pool.shape[0]
        if uniform:
            idx = torch.randint(0, M, (n_samples,), generator=gen, device=self.device)
            wts = torch.ones(n_samples, dtype=torch.float64, device=self.device)
        else:
            q = self.proposal(pool, r12s, r13s, mu, bf16=bf16)
            cdf = torch.cumsum(q, 0)
            u = torch.rand(n_samples, generator=gen, device=self.device, dtype=torch.float64) * cdf[-1]
            idx = torch.searchsorted(cdf, u).clamp_max(M - 1)
            wts = (1.0 / M) / q[idx]
        rs = np.random.RandomState(seed)
        off = rotation_offsets(r12s, r13s, mu, n_samples, rng=rs)
        # one rotation per sampled centre: evaluate f_k = n1 n2 n3 at (centre_k, rotation_k)
        cen = pool[idx]
        vals = torch.empty(n_samples, dtype=torch.float64, device=self.device)
        chunk = 1 << 20
        for s in range(0, n_samples, chunk):
            e = min(n_samples, s + chunk)
            vals[s:e] = self._f_pairs(cen[s:e], off[s:e])
        v = vals * wts
        return float(v.mean()), v

    def draw(self, q, n, generator):
        """n i.i.d. pool indices from q and their weights (1/M)/q_i."""
        M = q.shape[0]
        cdf = torch.cumsum(q, 0)
        u = torch.rand(n, generator=generator, device=self.device, dtype=torch.float64) * cdf[-1]
        idx = torch.searchsorted(cdf, u).clamp_max(M - 1)
        return idx, (1.0 / M) / q[idx]

    def sample_stats(self, pool, r12s, r13s, mu, n_samples, seed=0, uniform=False, bf16=True, q=None,
                     replicates=8):
        """Single-triplet estimate of the pool mean of E_rot[f] through
        hermes_mc_sample (rotations drawn on the GPU), as `replicates`
        independent runs of n_samples / replicates i.i.d. samples: uniform
        centres (weight 1) or centres from the proposal q (weight (1/M)/q).
        Returns (mean, standard error from the replicate spread, variance
        per sample)."""
        if not uniform and q is None:
            q = self.proposal(pool, r12s, r13s, mu, bf16=bf16)
        gen = torch.Generator(device=self.device).manual_seed(seed)
        nr = max(n_samples // replicates, 1)
        means, s1, s2 = [], 0.0, 0.0
        for r in range(replicates):
            rseed = (seed * 0x9E3779B97F4A7C15 + r * 0xBF58476D1CE4E5B9) & ((1 << 64) - 1)
            idx, wts = (None, None) if uniform else self.draw(q, nr, gen)
            a, b = mc_sample(self.e1, self.e2, self.e3, self.J, pool, self.phi_t, r12s, r13s, mu, nr, rseed,
                             idx=idx, weights=wts)
            means.append(a / nr)
            s1 += a
            s2 += b
        nt = nr * replicates
        mean = float(np.mean(means))
        var = max(s2 / nt - (s1 / nt) ** 2, 0.0)
        return mean, float(np.std(means, ddof=1) / np.sqrt(replicates)), var

    def centre_estimate(self, r12s, r13s, mu, n_centres, n_rot, seed=0, uniform=False, pool_factor=4,
                        replicates=8, bf16=True):
        """The reference estimator's form (centres x rotations, one rotation
        set per run from a seeded MT19937 as rotation_offsets) with the
        centres importance-sampled: each replicate draws a fresh uniform pool
        of pool_factor * n_centres candidates, evaluates the proposal on it,
        takes n_centres i.i.d. centres from q and weights them (1/M)/q, so
        the estimate is unbiased for the box mean of E_rot[f].  Uniform:
        n_centres uniform centres, weight 1.  Returns (mean, standard error
        from the replicate spread)."""
        gen = torch.Generator(device=self.device).manual_seed(seed)
        means = []
        for r in range(replicates):
            off = rotation_offsets(r12s, r13s, mu, n_rot, rng=np.random.RandomState((seed * 1000003 + r) % (1 << 31)))
            if uniform:
                cen = torch.rand((n_centres, 3), generator=gen, device=self.device, dtype=torch.float64) * self.L
                w = None
            else:
                pool = torch.rand((pool_factor * n_centres, 3), generator=gen, device=self.device,
                                  dtype=torch.float64) * self.L
                q = self.proposal(pool, r12s, r13s, mu, bf16=bf16)
                idx, w = self.draw(q, n_centres, gen)
                cen = pool[idx].contiguous()
            tot, _ = triplet_sum(self.e1, self.e2, self.e3, self.J, cen, off, self.phi_t, center_w=w)
            means.append(tot / (n_centres * n_rot))
        return float(np.mean(means)), float(np.std(means, ddof=1) / np.sqrt(replicates))

    def _f_pairs(self, centers, offsets):
        o = torch.as_tensor(offsets, device=self.device)
        n1 = interp(self.e1, self.J, centers, self.phi_t)
        n2 = interp(self.e2, self.J, centers + o[:, 0:3], self.phi_t)
        n3 = interp(self.e3, self.J, centers + o[:, 3:6], self.phi_t)
        return n1 * n2 * n3
